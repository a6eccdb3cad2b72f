// Per-element-type dispatch over (form, precision, DOFs per node).  One
// translation unit per element type instantiates it (forms_<type>.cu) so the
// build compiles them in parallel.
#pragma once

#include <cstdlib>

#include "elements.cuh"
#include "exact.cuh"
#include "mixed_fast.cuh"
#include "mixed_tc.cuh"

namespace fegpu {

// FP64 colour-ordered kernels (every form).  The mixed-precision path goes
// through launch_mixed_et (FP32 element blocks for the row gather).
template <int ET>
int launch_form_et(int form, int precision, int ndn, const KArgs &a, int sms, cudaStream_t s) {
  constexpr bool SOLID = ElemT<ET>::MDIM == 3;
  (void)precision;
  switch (form) {
    case F_DIFF_ISO: return launch_one<ET, F_DIFF_ISO, double, 1>(a, sms, s);
    case F_DIFF_GEN: return launch_one<ET, F_DIFF_GEN, double, 1>(a, sms, s);
    case F_ELAST_ISO:
      if constexpr (SOLID) return launch_one<ET, F_ELAST_ISO, double, 3>(a, sms, s);
      break;
    case F_ELAST_GEN:
      if constexpr (SOLID) return launch_one<ET, F_ELAST_GEN, double, 3>(a, sms, s);
      break;
    case F_DOT:
      if (ndn == 1) return launch_one<ET, F_DOT, double, 1>(a, sms, s);
      if (ndn == 2) return launch_one<ET, F_DOT, double, 2>(a, sms, s);
      if (ndn == 3) return launch_one<ET, F_DOT, double, 3>(a, sms, s);
      break;
    case F_LIN:
      if (ndn == 1) return launch_one<ET, F_LIN, double, 1>(a, sms, s);
      if (ndn == 2) return launch_one<ET, F_LIN, double, 2>(a, sms, s);
      if (ndn == 3) return launch_one<ET, F_LIN, double, 3>(a, sms, s);
      break;
  }
  throw Error{FEGPU_ERR_ARG, "form not available for this element type / DOF count"};
}

template <int ET>
int launch_mixed_et(int form, const KArgs &a, int sms, cudaStream_t s) {
  constexpr bool SOLID = ElemT<ET>::MDIM == 3;
  switch (form) {
    case F_DIFF_ISO: return launch_blocks_mixed_t<ET, F_DIFF_ISO, 1>(a, sms, s);
    case F_DIFF_GEN: return launch_blocks_mixed_t<ET, F_DIFF_GEN, 1>(a, sms, s);
    case F_ELAST_ISO:
      if constexpr (SOLID) {
        if (tc_enabled(a)) return launch_blocks_tc<ET>(a, sms, s);
        return launch_blocks_mixed_t<ET, F_ELAST_ISO, 3>(a, sms, s);
      }
      break;
    case F_ELAST_GEN:
      if constexpr (SOLID) return launch_blocks_mixed_t<ET, F_ELAST_GEN, 3>(a, sms, s);
      break;
  }
  throw Error{FEGPU_ERR_ARG, "mixed precision: form not available for this element type"};
}

// Reference-order FP64 element blocks (exact.cuh) for the row gather of exact.cu.
template <int ET>
int launch_exact_et(int form, const KArgs &a, int sms, cudaStream_t s) {
  constexpr bool SOLID = ElemT<ET>::MDIM == 3;
  switch (form) {
    case F_DIFF_ISO: return launch_blocks_exact_t<ET, F_DIFF_ISO>(a, sms, s);
    case F_DIFF_GEN: return launch_blocks_exact_t<ET, F_DIFF_GEN>(a, sms, s);
    case F_ELAST_ISO:
      if constexpr (SOLID) return launch_blocks_exact_t<ET, F_ELAST_ISO>(a, sms, s);
      break;
    case F_ELAST_GEN:
      if constexpr (SOLID) return launch_blocks_exact_t<ET, F_ELAST_GEN>(a, sms, s);
      break;
  }
  throw Error{FEGPU_ERR_ARG, "reference-order FP64: form not available for this element type"};
}

int launch_exact_q4(int, const KArgs &, int, cudaStream_t);
int launch_exact_h8(int, const KArgs &, int, cudaStream_t);
int launch_exact_h20(int, const KArgs &, int, cudaStream_t);
int launch_exact_t4(int, const KArgs &, int, cudaStream_t);
int launch_exact_t10(int, const KArgs &, int, cudaStream_t);
int launch_form_q4(int, int, int, const KArgs &, int, cudaStream_t);
int launch_form_h8(int, int, int, const KArgs &, int, cudaStream_t);
int launch_form_h20(int, int, int, const KArgs &, int, cudaStream_t);
int launch_form_t4(int, int, int, const KArgs &, int, cudaStream_t);
int launch_form_t10(int, int, int, const KArgs &, int, cudaStream_t);
int launch_mixed(int etype, int form, const KArgs &a, int sms, cudaStream_t s);
int launch_mixed_q4(int, const KArgs &, int, cudaStream_t);
int launch_mixed_h8(int, const KArgs &, int, cudaStream_t);
int launch_mixed_h20(int, const KArgs &, int, cudaStream_t);
int launch_mixed_t4(int, const KArgs &, int, cudaStream_t);
int launch_mixed_t10(int, const KArgs &, int, cudaStream_t);

}  // namespace fegpu
