// staged_inst.cu — instantiations of the staged half-steps for one PML kind (GBF_PK), compiled
// once per kind so the library builds in parallel.
#define GBF_KERNELS_ONLY
#include "staged.cuh"

#ifndef GBF_PK
#error "GBF_PK must be defined (0..4)"
#endif

namespace gbf {

#define GBF_CAT2(a, b) a##b
#define GBF_CAT(a, b) GBF_CAT2(a, b)

// The staged half-steps for PML kind GBF_PK: E for `np` poles (real or complex pole state), H
// for ID layout `idp` (0: the one H row of every material, 1: packed IDs); NULL where a staged
// form does not apply (more than two poles, three ID arrays per node): those models keep the
// plain kernels.
void GBF_CAT(staged_pk, GBF_PK)(int np, int treal, int idp, SKernFn* e, SKernFn* h) {
  switch (np) {
    case 0: *e = e_half_step_staged<GBF_PK, 0, false>; break;
    case 1: *e = treal ? e_half_step_staged<GBF_PK, 1, true> : e_half_step_staged<GBF_PK, 1, false>; break;
    case 2: *e = treal ? e_half_step_staged<GBF_PK, 2, true> : e_half_step_staged<GBF_PK, 2, false>; break;
    default: *e = nullptr; break;
  }
  *h = idp == 0 ? h_half_step_staged<GBF_PK, 0> : idp == 1 ? h_half_step_staged<GBF_PK, 1> : nullptr;
}

}  // namespace gbf
