// status.h -- the library's internal error type: raised inside, converted
// into a status code and the per-thread last-error string at the C ABI.
// No CUDA dependency, so host-only sources (the generators) can use it.
#pragma once

#include <stdexcept>
#include <string>

#include "gpuh2h.h"

namespace gh {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define GH_CHECK(cond, code, msg)                 \
  do {                                            \
    if (!(cond)) throw ::gh::Error((code), (msg)); \
  } while (0)

}  // namespace gh
