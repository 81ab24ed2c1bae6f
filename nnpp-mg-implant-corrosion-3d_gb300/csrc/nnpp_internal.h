// nnpp_internal.h -- declarations shared by the host C++ and the CUDA translation units.
#ifndef NNPP_INTERNAL_H
#define NNPP_INTERNAL_H

#include <cstdint>
#include <string>

#include "nnpp_gb300.h"

namespace nnpp {

// Thread-local last-error message; returns st for chaining.
nnpp_status set_error(nnpp_status st, const std::string& msg);
void clear_error();

void synth_default_params(int n_side, nnpp_params* p);

}  // namespace nnpp

#endif  // NNPP_INTERNAL_H
