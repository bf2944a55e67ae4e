/* Minimal stand-in for glog's logging macros, used only to compile the
 * reference's radix helpers into the test oracle (oracle/_ref).  Every
 * macro discards its stream. */
#ifndef GBJ_SHIM_GLOG_LOGGING_H
#define GBJ_SHIM_GLOG_LOGGING_H
#include <ostream>
namespace gbj_shim {
struct NullStream : std::ostream {
  NullStream() : std::ostream(nullptr) {}
};
inline NullStream &null_stream() {
  static thread_local NullStream s;
  return s;
}
}  // namespace gbj_shim
#define LOG(sev) ::gbj_shim::null_stream()
#define VLOG(lvl) ::gbj_shim::null_stream()
#define LOG_IF(sev, cond) ::gbj_shim::null_stream()
#define VLOG_IF(lvl, cond) ::gbj_shim::null_stream()
#define CHECK(cond) ::gbj_shim::null_stream()
#endif
