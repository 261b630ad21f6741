// fused_inst.cu — instantiations of the fused step kernel for one PML kind (GBF_PK) and one
// tile height (GBF_TJ), compiled once per pair so the library builds in parallel.
#define GBF_KERNELS_ONLY
#include "fused_step.cuh"

#if !defined(GBF_PK) || !defined(GBF_TJ)
#error "GBF_PK (0..4) and GBF_TJ must be defined"
#endif

namespace gbf {

#define GBF_CAT4(a, b, c, d) a##b##c##d
#define GBF_NAME(a, b, c, d) GBF_CAT4(a, b, c, d)

template <int IDPH>
static FusedFn fused_for(int np, int treal) {
  switch (np) {
    case 0: return fused_step<GBF_PK, 0, false, IDPH, GBF_TJ>;
    case 1: return treal ? fused_step<GBF_PK, 1, true, IDPH, GBF_TJ>
                         : fused_step<GBF_PK, 1, false, IDPH, GBF_TJ>;
    case 2: return treal ? fused_step<GBF_PK, 2, true, IDPH, GBF_TJ>
                         : fused_step<GBF_PK, 2, false, IDPH, GBF_TJ>;
    default: return nullptr;   // more poles: the two half-step kernels
  }
}

// The fused step kernel for PML kind GBF_PK, tile height GBF_TJ, `np` poles (real state with
// `treal`) and, with `uniform_h`, the one H row shared by every material (no H IDs read).
FusedFn GBF_NAME(fused_kernel_pk, GBF_PK, _tj, GBF_TJ)(int np, int uniform_h, int treal) {
  return uniform_h ? fused_for<0>(np, treal) : fused_for<1>(np, treal);
}

}  // namespace gbf
