// Element kernels for FEGPU_T4: FP64 colour kernels, reference-order FP64
// blocks and FP32 block kernels.
#include "forms_dispatch.cuh"

namespace fegpu {
int launch_form_t4(int form, int precision, int ndn, const KArgs &a, int sms, cudaStream_t s) {
  return launch_form_et<FEGPU_T4>(form, precision, ndn, a, sms, s);
}
int launch_mixed_t4(int form, const KArgs &a, int sms, cudaStream_t s) {
  return launch_mixed_et<FEGPU_T4>(form, a, sms, s);
}
int launch_exact_t4(int form, const KArgs &a, int sms, cudaStream_t s) {
  return launch_exact_et<FEGPU_T4>(form, a, sms, s);
}
}  // namespace fegpu
