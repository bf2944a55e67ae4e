/* Stand-in for the reference's platform umbrella header, used only to
 * compile its radix helpers into the test oracle (oracle/_ref). */
#ifndef GBJ_SHIM_COMMON_HPP
#define GBJ_SHIM_COMMON_HPP
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <glog/logging.h>
#endif
