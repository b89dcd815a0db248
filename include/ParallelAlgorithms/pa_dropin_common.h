// Shared helper of the drop-in C++ headers in this directory: turns a
// pa_status from the C ABI (pa_gpu.h) into the exception a C++ caller of the
// reference would see.  The reference signals no errors of its own; its only
// failure mode is std::bad_alloc from operator new, which PA_ERR_OOM maps to.
#ifndef PA_DROPIN_COMMON_H
#define PA_DROPIN_COMMON_H

#include <new>
#include <stdexcept>
#include <string>

#include "../pa_gpu.h"

namespace ParallelAlgorithms {
namespace pa_detail {

inline void check(int status, const char* what) {
  if (status == PA_OK) return;
  if (status == PA_ERR_OOM) throw std::bad_alloc();
  std::string msg = std::string(what) + ": " + pa_status_string(status) + ": " + pa_last_error_message();
  if (status == PA_ERR_ARG) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

}  // namespace pa_detail
}  // namespace ParallelAlgorithms

#endif  // PA_DROPIN_COMMON_H
