// errors.cpp -- thread-local error message of the C ABI.
#include <string>

#include "nnpp_internal.h"

namespace nnpp {

namespace {
thread_local std::string g_last_error;
}

nnpp_status set_error(nnpp_status st, const std::string& msg) {
  if (st != NNPP_OK) g_last_error = msg;
  return st;
}

void clear_error() { g_last_error.clear(); }

}  // namespace nnpp

extern "C" const char* nnpp_last_error(void) { return nnpp::g_last_error.c_str(); }

extern "C" int nnpp_abi_version(void) { return NNPP_ABI_VERSION; }
