// Element kernels for FEGPU_H8: FP64 colour kernels, reference-order FP64
// blocks and FP32 block kernels.
#include "forms_dispatch.cuh"

namespace fegpu {
int launch_form_h8(int form, int precision, int ndn, const KArgs &a, int sms, cudaStream_t s) {
  return launch_form_et<FEGPU_H8>(form, precision, ndn, a, sms, s);
}
int launch_mixed_h8(int form, const KArgs &a, int sms, cudaStream_t s) {
  return launch_mixed_et<FEGPU_H8>(form, a, sms, s);
}
int launch_exact_h8(int form, const KArgs &a, int sms, cudaStream_t s) {
  return launch_exact_et<FEGPU_H8>(form, a, sms, s);
}
}  // namespace fegpu
