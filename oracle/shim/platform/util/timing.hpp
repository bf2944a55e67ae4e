/* Stand-in for the reference's RAII timer, used only to compile its radix
 * helpers into the test oracle (oracle/_ref).  It measures nothing. */
#ifndef GBJ_SHIM_TIMING_HPP
#define GBJ_SHIM_TIMING_HPP
#include <string>
class time_block {
 public:
  explicit time_block(const std::string &) {}
  explicit time_block(const char *) {}
};
#endif
