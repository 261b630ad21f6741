// staged_inst.cu — instantiations of the staged E half-step for one PML kind (GBF_PK), compiled
// once per kind so the library builds in parallel.
#define GBF_KERNELS_ONLY
#include "staged_e.cuh"

#ifndef GBF_PK
#error "GBF_PK must be defined (0..4)"
#endif

namespace gbf {

#define GBF_CAT2(a, b) a##b
#define GBF_CAT(a, b) GBF_CAT2(a, b)

// The staged E half-step for PML kind GBF_PK and `np` poles, or NULL where it does not apply
// (complex pole state, more than two poles): those models keep the plain kernel.
void GBF_CAT(staged_pk, GBF_PK)(int np, int treal, SKernFn* e) {
  switch (np) {
    case 0: *e = e_half_step_staged<GBF_PK, 0, false>; break;
    case 1: *e = treal ? e_half_step_staged<GBF_PK, 1, true> : nullptr; break;
    case 2: *e = treal ? e_half_step_staged<GBF_PK, 2, true> : nullptr; break;
    default: *e = nullptr; break;
  }
}

}  // namespace gbf
