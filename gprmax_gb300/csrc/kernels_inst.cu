// kernels_inst.cu — instantiations of the half-step kernels for one PML kind (GBF_PK), compiled
// once per kind so the library builds in parallel.
#define GBF_KERNELS_ONLY
#include "fdtd_kernels.cuh"

#ifndef GBF_PK
#error "GBF_PK must be defined (0..4)"
#endif

namespace gbf {

#define GBF_CAT2(a, b) a##b
#define GBF_CAT(a, b) GBF_CAT2(a, b)

template <int IDP, bool TR>
static EKernFn e_for(int np) {
  switch (np) {
    case 1: return e_half_step<GBF_PK, 1, IDP, TR>;
    case 2: return e_half_step<GBF_PK, 2, IDP, TR>;
    case 3: return e_half_step<GBF_PK, 3, IDP, TR>;
    case 4: return e_half_step<GBF_PK, 4, IDP, TR>;
    default: return e_half_step<GBF_PK, 0, IDP, false>;
  }
}

// Kernels for PML kind GBF_PK, `np` dispersive poles and ID layout `idp` (1 packed, 3 plain);
// with `uniform_h` the H half-step takes the one H row of every material (no IDs); with `treal`
// (packed IDs only) the dispersive state is stored as real parts.
void GBF_CAT(kernels_pk, GBF_PK)(int np, int idp, int uniform_h, int treal, HKernFn* h,
                                 EKernFn* e) {
  if (idp == 1) {
    *h = h_half_step<GBF_PK, 1>;
    *e = treal ? e_for<1, true>(np) : e_for<1, false>(np);
  } else {
    *h = h_half_step<GBF_PK, 3>;
    *e = e_for<3, false>(np);
  }
  if (uniform_h) *h = h_half_step<GBF_PK, 0>;
}

template <int IDP, bool TR>
static BKernFn eb_for(int np) {
  switch (np) {
    case 1: return e_half_step_batch<GBF_PK, 1, IDP, TR>;
    case 2: return e_half_step_batch<GBF_PK, 2, IDP, TR>;
    case 3: return e_half_step_batch<GBF_PK, 3, IDP, TR>;
    case 4: return e_half_step_batch<GBF_PK, 4, IDP, TR>;
    default: return e_half_step_batch<GBF_PK, 0, IDP, false>;
  }
}

// Batched kernels for PML kind GBF_PK (see kernels_pk*).
void GBF_CAT(batch_kernels_pk, GBF_PK)(int np, int idp, int uniform_h, int treal, BKernFn* h,
                                       BKernFn* e) {
  if (idp == 1) {
    *h = h_half_step_batch<GBF_PK, 1>;
    *e = treal ? eb_for<1, true>(np) : eb_for<1, false>(np);
  } else {
    *h = h_half_step_batch<GBF_PK, 3>;
    *e = eb_for<3, false>(np);
  }
  if (uniform_h) *h = h_half_step_batch<GBF_PK, 0>;
}

}  // namespace gbf
