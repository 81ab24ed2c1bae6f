// pending.cu -- entry points whose implementation is not in this build yet.
#include "handle.cuh"

using namespace nnpp;

extern "C" {
nnpp_status nnpp_forward_ckpt(nnpp_handle*, int, int, int, int, double*) {
  return set_error(NNPP_ERR_UNSUPPORTED, "forward_ckpt: not available in this build");
}
nnpp_status nnpp_backward(nnpp_handle*, const double*, double*, double*) {
  return set_error(NNPP_ERR_UNSUPPORTED, "backward: not available in this build");
}
nnpp_status nnpp_ensemble_create(nnpp_ensemble**, nnpp_handle* const*, int) {
  return set_error(NNPP_ERR_UNSUPPORTED, "ensembles: not available in this build");
}
nnpp_status nnpp_ensemble_forward(nnpp_ensemble*, int, int) {
  return set_error(NNPP_ERR_UNSUPPORTED, "ensembles: not available in this build");
}
nnpp_status nnpp_ensemble_destroy(nnpp_ensemble*) { return NNPP_OK; }
}
