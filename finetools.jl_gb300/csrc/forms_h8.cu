// Element kernels for FEGPU_H8 (all forms, both precisions).
#include "forms_dispatch.cuh"

namespace fegpu {
int launch_form_h8(int form, int precision, int ndn, const KArgs &a, int sms, cudaStream_t s) {
  return launch_form_et<FEGPU_H8>(form, precision, ndn, a, sms, s);
}
}  // namespace fegpu
