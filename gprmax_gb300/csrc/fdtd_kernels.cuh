// fdtd_kernels.cuh — fused Yee half-step kernels for sm_103a.
//
// One H kernel and one E kernel advance a whole time step. Each kernel touches every field
// value, material ID and PML/dispersive state word it needs once per half-step:
//
//   H half-step  (gprMax/fields_updates_ext.pyx:352-412 update_magnetic, then the six
//                 pml_updates_magnetic_*_ext.pyx slab corrections in slab order, then the
//                 magnetic-dipole sources, model_build_run.py:434-442)
//   E half-step  (update_electric :30-110 or update_electric_dispersive_*_A :113-297, the six
//                 pml_updates_electric_*_ext.pyx corrections, the voltage-source and
//                 Hertzian-dipole sources, and the dispersive part B :183-349 with the final E,
//                 model_build_run.py:444-470)
//
// The arithmetic of each term is the reference's, in the reference's order: the main update
// first, then each slab's additive correction in slab order x0, y0, z0, xmax, ymax, zmax, then
// the sources. Only the schedule differs: the corrections are applied in registers by the
// thread that owns the node instead of by separate passes over the slabs.
//
// Thread mapping: a block covers 32 consecutive k (one warp per row) by BY rows j, and walks
// a chunk of x planes; the previous plane's H (E kernel) or the next plane's E (H kernel) stays
// in registers, so each plane of the marching field is read from memory once per block.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbf {

constexpr int kBX = 32;   // k extent of a block (one warp)
constexpr int kBY = 8;    // j extent of a block
constexpr int kMaxPoles = 4;

// PML kinds: formulation x order (pml.py:156-159 and len(G.cfs))
enum PmlKind : int { PML_NONE = 0, PML_HORI1 = 1, PML_HORI2 = 2, PML_MRI1 = 3, PML_MRI2 = 4 };

struct Slab {
  int axis;         // 0 x, 1 y, 2 z
  int minus;        // 1 for x0 / y0 / z0 (profile index counts down towards the boundary)
  int T;            // thickness in cells
  int n_axis;       // nx, ny or nz
  int nu, nv;       // extents of the two other axes (cells) used to index Phi
  float d;          // cell size along the axis (fp32, the kernels' `float d`)
  long long ocount; // Phi elements per CFS order
  float* phiE1;     // Phi arrays [order][...]: E first/second tangential component
  float* phiE2;
  float* phiH1;
  float* phiH2;
  const float* eR;  // [4][order][T]: RA, RB, RE, RF for E
  const float* hR;  // same for H
};

struct Src {
  int kind, comp, i, j, k, first, last, pad;
  float s0, s1;
  const float* w;   // this source's waveform table [iterations]
};

struct StepParams {
  float* E[3];
  float* H[3];
  const uint32_t* ID;     // [6][ncomp]
  long long ncomp;        // nodes per component
  int nx, ny, nz;
  int sy, sx;             // strides: j -> nz+1, i -> (ny+1)(nz+1)  (sx fits int for < 2^31 nodes)
  const float* cE;        // [nmat][5]
  const float* cH;        // [nmat][5]
  const float2* cD;       // [nmat][3P]
  float2* T;              // [3][P][ncomp]
  int P;
  int nslab;
  Slab slab[6];
  int nsrcE, nsrcH;
  const Src* srcE;
  const Src* srcH;
  const int* d_it;
  int chunk;              // x planes per block
};

// ---------------------------------------------------------------------------------------
// CFS-PML correction of one field value (pml_updates_{electric,magnetic}_{HORIPML,MRIPML}).
// Returns X such that the field changes by (+/-) c4 * X, and advances the Phi recursion.
// RA01, IRA, RC0 ... are recomputed from the stored rows exactly as the reference does per i.
template <int PK>
__device__ __forceinline__ float pml_term(float dF, float* phi, long long pidx, long long ocount,
                                          const float* __restrict__ R, int order, int T, int p) {
  const float RA0 = __ldg(R + (0 * order + 0) * T + p);
  const float RB0 = __ldg(R + (1 * order + 0) * T + p);
  const float RE0 = __ldg(R + (2 * order + 0) * T + p);
  const float RF0 = __ldg(R + (3 * order + 0) * T + p);
  float ph0 = phi[pidx];
  if (PK == PML_HORI1) {
    const float RA01 = RA0 - 1.0f;
    const float X = RA01 * dF + RB0 * ph0;
    phi[pidx] = RE0 * ph0 - RF0 * dF;
    return X;
  } else if (PK == PML_HORI2) {
    const float RA1 = __ldg(R + (0 * order + 1) * T + p);
    const float RB1 = __ldg(R + (1 * order + 1) * T + p);
    const float RE1 = __ldg(R + (2 * order + 1) * T + p);
    const float RF1 = __ldg(R + (3 * order + 1) * T + p);
    const float RA01 = RA0 * RA1 - 1.0f;
    float ph1 = phi[pidx + ocount];
    const float X = RA01 * dF + RA1 * RB0 * ph0 + RB1 * ph1;
    phi[pidx + ocount] = RE1 * ph1 - RF1 * (RA0 * dF + RB0 * ph0);
    phi[pidx] = RE0 * ph0 - RF0 * dF;
    return X;
  } else if (PK == PML_MRI1) {
    const float IRA = 1.0f / RA0;
    const float IRA1 = IRA - 1.0f;
    const float RC0 = IRA * RB0 * RF0;
    const float X = IRA1 * dF - IRA * ph0;
    phi[pidx] = RE0 * ph0 + RC0 * dF - RC0 * ph0;
    return X;
  } else {  // PML_MRI2
    const float RA1 = __ldg(R + (0 * order + 1) * T + p);
    const float RB1 = __ldg(R + (1 * order + 1) * T + p);
    const float RE1 = __ldg(R + (2 * order + 1) * T + p);
    const float RF1 = __ldg(R + (3 * order + 1) * T + p);
    const float IRA = 1.0f / (RA0 + RA1);
    const float IRA1 = IRA - 1.0f;
    const float RC0 = IRA * RF0;
    const float RC1 = IRA * RF1;
    float ph1 = phi[pidx + ocount];
    const float Psi = RB0 * ph0 + RB1 * ph1;
    const float X = IRA1 * dF - IRA * Psi;
    phi[pidx + ocount] = RE1 * ph1 + RC1 * (dF - Psi);
    phi[pidx] = RE0 * ph0 + RC0 * (dF - Psi);
    return X;
  }
}

// Phi index of node (i, j, k) in a slab at profile index p (layouts: x [p][j][k],
// y [i][p][k], z [i][j][p]).
__device__ __forceinline__ long long phi_index(const Slab& s, int i, int j, int k, int p) {
  if (s.axis == 0) return ((long long)p * s.nu + j) * s.nv + k;
  if (s.axis == 1) return ((long long)i * s.T + p) * s.nv + k;
  return ((long long)i * s.nv + j) * s.T + p;
}

// ---------------------------------------------------------------------------------------
// H half-step. Domain: i in [0, nx], j in [0, ny], k in [0, nz].
template <int PK>
__global__ void __launch_bounds__(kBX * kBY)
h_half_step(const StepParams p) {
  const int k = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (k > p.nz || j > p.ny) return;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int i0 = blockIdx.z * p.chunk;
  const int i1 = min(i0 + p.chunk, nx + 1);
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  float* Hx = p.H[0];
  float* Hy = p.H[1];
  float* Hz = p.H[2];
  const int it = *p.d_it;
  const bool jin = j < ny, kin = k < nz;
  const int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;

  // E of plane i (own node) is carried from the previous iteration's "next plane" loads
  long long idx = (long long)i0 * p.sx + (long long)j * p.sy + k;
  float ey_c = __ldg(Ey + idx), ez_c = __ldg(Ez + idx);
  for (int i = i0; i < i1; ++i, idx += p.sx) {
    const float ex_c = __ldg(Ex + idx);
    const float ex_j = jin ? __ldg(Ex + idx + p.sy) : 0.f;
    const float ez_j = jin ? __ldg(Ez + idx + p.sy) : 0.f;
    const float ex_k = kin ? __ldg(Ex + idx + 1) : 0.f;
    const float ey_k = kin ? __ldg(Ey + idx + 1) : 0.f;
    float ey_n = 0.f, ez_n = 0.f;
    if (i < nx) {
      ey_n = __ldg(Ey + idx + p.sx);
      ez_n = __ldg(Ez + idx + p.sx);
    }
    const float dEz_y = ez_j - ez_c;   // Hx main and y-slab
    const float dEy_z = ey_k - ey_c;   // Hx main and z-slab
    const float dEx_z = ex_k - ex_c;   // Hy main and z-slab
    const float dEz_x = ez_n - ez_c;   // Hy main and x-slab
    const float dEy_x = ey_n - ey_c;   // Hz main and x-slab
    const float dEx_y = ex_j - ex_c;   // Hz main and y-slab

    // --- Hx: main i in [1,nx], j in [0,ny), k in [0,nz)
    {
      const bool mainu = (i >= 1) && jin && kin;
      bool pml = false;
      if (PK != PML_NONE && i < nx && jin && kin) {
        for (int s = 0; s < p.nslab; ++s) {
          const Slab& sl = p.slab[s];
          if (sl.axis == 0) continue;
          const int c = sl.axis == 1 ? j : k;
          if (sl.minus ? (c < sl.T) : (c >= sl.n_axis - sl.T)) pml = true;
        }
      }
      bool src = false;
      for (int s = 0; s < p.nsrcH; ++s) {
        const Src& q = p.srcH[s];
        if (q.comp == 3 && q.i == i && q.j == j && q.k == k) src = true;
      }
      if (mainu || pml || src) {
        const uint32_t m = __ldg(p.ID + 3 * p.ncomp + idx);
        const float* c = p.cH + 5 * (long long)m;
        float F = Hx[idx];
        if (mainu) F = __ldg(c + 0) * F - __ldg(c + 2) * dEz_y + __ldg(c + 3) * dEy_z;
        if (PK != PML_NONE && pml) {
          const float c4 = __ldg(c + 4);
          for (int s = 0; s < p.nslab; ++s) {
            const Slab& sl = p.slab[s];
            if (sl.axis == 0) continue;
            const int cc = sl.axis == 1 ? j : k;
            if (!(sl.minus ? (cc < sl.T) : (cc >= sl.n_axis - sl.T))) continue;
            const int pp = sl.minus ? (sl.T - 1 - cc) : (cc - (sl.n_axis - sl.T));
            const long long pi = phi_index(sl, i, j, k, pp);
            if (sl.axis == 1) {  // y-slab: Phi1, dEz/dy, Hx -= c4*X
              const float X = pml_term<PK>(dEz_y / sl.d, sl.phiH1, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F - c4 * X;
            } else {             // z-slab: Phi1, dEy/dz, Hx += c4*X
              const float X = pml_term<PK>(dEy_z / sl.d, sl.phiH1, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F + c4 * X;
            }
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 3 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(__ldg(c + 4), __ldg(q.w + it)), q.s0));
          }
        }
        Hx[idx] = F;
      }
    }
    // --- Hy: main i in [0,nx), j in [1,ny], k in [0,nz)
    {
      const bool mainu = (i < nx) && (j >= 1) && kin;
      bool pml = false;
      if (PK != PML_NONE && i < nx && jin && kin) {
        for (int s = 0; s < p.nslab; ++s) {
          const Slab& sl = p.slab[s];
          if (sl.axis == 1) continue;
          const int c = sl.axis == 0 ? i : k;
          if (sl.minus ? (c < sl.T) : (c >= sl.n_axis - sl.T)) pml = true;
        }
      }
      bool src = false;
      for (int s = 0; s < p.nsrcH; ++s) {
        const Src& q = p.srcH[s];
        if (q.comp == 4 && q.i == i && q.j == j && q.k == k) src = true;
      }
      if (mainu || pml || src) {
        const uint32_t m = __ldg(p.ID + 4 * p.ncomp + idx);
        const float* c = p.cH + 5 * (long long)m;
        float F = Hy[idx];
        if (mainu) F = __ldg(c + 0) * F - __ldg(c + 3) * dEx_z + __ldg(c + 1) * dEz_x;
        if (PK != PML_NONE && pml) {
          const float c4 = __ldg(c + 4);
          for (int s = 0; s < p.nslab; ++s) {
            const Slab& sl = p.slab[s];
            if (sl.axis == 1) continue;
            const int cc = sl.axis == 0 ? i : k;
            if (!(sl.minus ? (cc < sl.T) : (cc >= sl.n_axis - sl.T))) continue;
            const int pp = sl.minus ? (sl.T - 1 - cc) : (cc - (sl.n_axis - sl.T));
            const long long pi = phi_index(sl, i, j, k, pp);
            if (sl.axis == 0) {  // x-slab: Phi1, dEz/dx, Hy += c4*X
              const float X = pml_term<PK>(dEz_x / sl.d, sl.phiH1, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F + c4 * X;
            } else {             // z-slab: Phi2, dEx/dz, Hy -= c4*X
              const float X = pml_term<PK>(dEx_z / sl.d, sl.phiH2, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F - c4 * X;
            }
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 4 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(__ldg(c + 4), __ldg(q.w + it)), q.s0));
          }
        }
        Hy[idx] = F;
      }
    }
    // --- Hz: main i in [0,nx), j in [0,ny), k in [1,nz]
    {
      const bool mainu = (i < nx) && jin && (k >= 1);
      bool pml = false;
      if (PK != PML_NONE && i < nx && jin && kin) {
        for (int s = 0; s < p.nslab; ++s) {
          const Slab& sl = p.slab[s];
          if (sl.axis == 2) continue;
          const int c = sl.axis == 0 ? i : j;
          if (sl.minus ? (c < sl.T) : (c >= sl.n_axis - sl.T)) pml = true;
        }
      }
      bool src = false;
      for (int s = 0; s < p.nsrcH; ++s) {
        const Src& q = p.srcH[s];
        if (q.comp == 5 && q.i == i && q.j == j && q.k == k) src = true;
      }
      if (mainu || pml || src) {
        const uint32_t m = __ldg(p.ID + 5 * p.ncomp + idx);
        const float* c = p.cH + 5 * (long long)m;
        float F = Hz[idx];
        if (mainu) F = __ldg(c + 0) * F - __ldg(c + 1) * dEy_x + __ldg(c + 2) * dEx_y;
        if (PK != PML_NONE && pml) {
          const float c4 = __ldg(c + 4);
          for (int s = 0; s < p.nslab; ++s) {
            const Slab& sl = p.slab[s];
            if (sl.axis == 2) continue;
            const int cc = sl.axis == 0 ? i : j;
            if (!(sl.minus ? (cc < sl.T) : (cc >= sl.n_axis - sl.T))) continue;
            const int pp = sl.minus ? (sl.T - 1 - cc) : (cc - (sl.n_axis - sl.T));
            const long long pi = phi_index(sl, i, j, k, pp);
            if (sl.axis == 0) {  // x-slab: Phi2, dEy/dx, Hz -= c4*X
              const float X = pml_term<PK>(dEy_x / sl.d, sl.phiH2, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F - c4 * X;
            } else {             // y-slab: Phi2, dEx/dy, Hz += c4*X
              const float X = pml_term<PK>(dEx_y / sl.d, sl.phiH2, pi, sl.ocount, sl.hR, order, sl.T, pp);
              F = F + c4 * X;
            }
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 5 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(__ldg(c + 4), __ldg(q.w + it)), q.s0));
          }
        }
        Hz[idx] = F;
      }
    }
    ey_c = ey_n;
    ez_c = ez_n;
  }
}

// ---------------------------------------------------------------------------------------
// Electric sources at one node/component, in list order (voltage sources, then Hertzian
// dipoles): sources.py:81-120 and :163-193 with numpy-2 fp32 operation order.
__device__ __forceinline__ float apply_e_sources(float F, int comp, int i, int j, int k, int it,
                                                 float c4, const StepParams& p) {
  for (int s = 0; s < p.nsrcE; ++s) {
    const Src& q = p.srcE[s];
    if (q.comp != comp || q.i != i || q.j != j || q.k != k) continue;
    if (it < q.first || it > q.last) continue;
    const float w = __ldg(q.w + it);
    if (q.kind == 0) {        // Hertzian dipole
      F = __fsub_rn(F, __fmul_rn(__fmul_rn(__fmul_rn(c4, w), q.s0), q.s1));
    } else if (q.kind == 1) { // resistive voltage source
      F = __fsub_rn(F, __fmul_rn(__fmul_rn(c4, w), q.s0));
    } else {                  // hard voltage source
      F = __fdiv_rn(-w, q.s0);
    }
  }
  return F;
}

// E half-step. Domain: i in [0, nx), j in [0, ny), k in [0, nz).
// NP = dispersive poles (0: non-dispersive).
template <int PK, int NP>
__global__ void __launch_bounds__(kBX * kBY)
e_half_step(const StepParams p) {
  const int k = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int nx = p.nx;
  const int i0 = blockIdx.z * p.chunk;
  const int i1 = min(i0 + p.chunk, nx);
  const float* __restrict__ Hx = p.H[0];
  const float* __restrict__ Hy = p.H[1];
  const float* __restrict__ Hz = p.H[2];
  const int it = *p.d_it;
  const int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  bool has_src = false;
  for (int s = 0; s < p.nsrcE; ++s) {
    const Src& q = p.srcE[s];
    if (q.j == j && q.k == k && q.i >= i0 && q.i < i1) has_src = true;
  }

  long long idx = (long long)i0 * p.sx + (long long)j * p.sy + k;
  float hy_p = 0.f, hz_p = 0.f;   // H of plane i-1
  if (i0 >= 1) {
    hy_p = __ldg(Hy + idx - p.sx);
    hz_p = __ldg(Hz + idx - p.sx);
  }
  for (int i = i0; i < i1; ++i, idx += p.sx) {
    const float hx_c = __ldg(Hx + idx), hy_c = __ldg(Hy + idx), hz_c = __ldg(Hz + idx);
    float hx_j = 0.f, hz_j = 0.f, hx_k = 0.f, hy_k = 0.f;
    if (j >= 1) { hx_j = __ldg(Hx + idx - p.sy); hz_j = __ldg(Hz + idx - p.sy); }
    if (k >= 1) { hx_k = __ldg(Hx + idx - 1); hy_k = __ldg(Hy + idx - 1); }
    const float dHz_y = hz_c - hz_j;   // Ex main and y-slab
    const float dHy_z = hy_c - hy_k;   // Ex main and z-slab
    const float dHx_z = hx_c - hx_k;   // Ey main and z-slab
    const float dHz_x = hz_c - hz_p;   // Ey main and x-slab
    const float dHy_x = hy_c - hy_p;   // Ez main and x-slab
    const float dHx_y = hx_c - hx_j;   // Ez main and y-slab
    const bool src_here = has_src;

#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      bool mainu;
      if (comp == 0) mainu = (j >= 1) && (k >= 1);
      else if (comp == 1) mainu = (i >= 1) && (k >= 1);
      else mainu = (i >= 1) && (j >= 1);
      bool pml = false;
      if (PK != PML_NONE) {
        for (int s = 0; s < p.nslab; ++s) {
          const Slab& sl = p.slab[s];
          if (sl.axis == comp) continue;
          const int c = sl.axis == 0 ? i : (sl.axis == 1 ? j : k);
          if (sl.minus ? (c >= 1 && c <= sl.T) : (c >= sl.n_axis - sl.T)) pml = true;
        }
      }
      if (!(mainu || pml || src_here)) continue;
      float* E = p.E[comp];
      const uint32_t m = __ldg(p.ID + comp * p.ncomp + idx);
      const float* c = p.cE + 5 * (long long)m;
      const float Eold = E[idx];
      float F = Eold;
      float2 TA[NP > 0 ? NP : 1];
      if (mainu) {
        // curl terms in the reference's order: CA*E + CB1*d1 - CB2*d2
        float t1, t2;
        const float CA = __ldg(c + 0);
        if (comp == 0) { t1 = __ldg(c + 2) * dHz_y; t2 = __ldg(c + 3) * dHy_z; }
        else if (comp == 1) { t1 = __ldg(c + 3) * dHx_z; t2 = __ldg(c + 1) * dHz_x; }
        else { t1 = __ldg(c + 1) * dHy_x; t2 = __ldg(c + 2) * dHx_y; }
        if (NP == 0) {
          F = CA * Eold + t1 - t2;
        } else {
          float phi = 0.f;
          const float2* cd = p.cD + (long long)m * 3 * NP;
          float2* Tc = p.T + (long long)comp * NP * p.ncomp + idx;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const float2 Tq = Tc[q * p.ncomp];
            const float2 a = __ldg(cd + 3 * q + 0);
            const float2 b = __ldg(cd + 3 * q + 1);
            const float2 z = __ldg(cd + 3 * q + 2);
            phi = phi + a.x * Tq.x;
            TA[q].x = (b.x * Tq.x - b.y * Tq.y) + z.x * Eold;
            TA[q].y = (b.x * Tq.y + b.y * Tq.x) + z.y * Eold;
          }
          F = CA * Eold + t1 - t2 - __ldg(c + 4) * phi;
        }
      }
      if (PK != PML_NONE && pml) {
        const float c4 = __ldg(c + 4);
        for (int s = 0; s < p.nslab; ++s) {
          const Slab& sl = p.slab[s];
          if (sl.axis == comp) continue;
          const int cc = sl.axis == 0 ? i : (sl.axis == 1 ? j : k);
          if (!(sl.minus ? (cc >= 1 && cc <= sl.T) : (cc >= sl.n_axis - sl.T))) continue;
          const int pp = sl.minus ? (sl.T - cc) : (cc - (sl.n_axis - sl.T));
          const long long pi = phi_index(sl, i, j, k, pp);
          // (component, slab axis) -> difference, Phi array and sign (see the header table)
          float dF; float* ph; float sgn;
          if (sl.axis == 0) {        // x-slab: Ey (Phi1, dHz/dx, -), Ez (Phi2, dHy/dx, +)
            if (comp == 1) { dF = dHz_x; ph = sl.phiE1; sgn = -1.f; }
            else { dF = dHy_x; ph = sl.phiE2; sgn = 1.f; }
          } else if (sl.axis == 1) { // y-slab: Ex (Phi1, dHz/dy, +), Ez (Phi2, dHx/dy, -)
            if (comp == 0) { dF = dHz_y; ph = sl.phiE1; sgn = 1.f; }
            else { dF = dHx_y; ph = sl.phiE2; sgn = -1.f; }
          } else {                   // z-slab: Ex (Phi1, dHy/dz, -), Ey (Phi2, dHx/dz, +)
            if (comp == 0) { dF = dHy_z; ph = sl.phiE1; sgn = -1.f; }
            else { dF = dHx_z; ph = sl.phiE2; sgn = 1.f; }
          }
          const float X = pml_term<PK>(dF / sl.d, ph, pi, sl.ocount, sl.eR, order, sl.T, pp);
          F = (sgn > 0.f) ? (F + c4 * X) : (F - c4 * X);
        }
      }
      if (src_here) F = apply_e_sources(F, comp, i, j, k, it, __ldg(c + 4), p);
      E[idx] = F;
      if (NP > 0 && mainu) {
        const float2* cd = p.cD + (long long)m * 3 * NP;
        float2* Tc = p.T + (long long)comp * NP * p.ncomp + idx;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float2 z = __ldg(cd + 3 * q + 2);
          float2 o;
          o.x = TA[q].x - z.x * F;
          o.y = TA[q].y - z.y * F;
          Tc[q * p.ncomp] = o;
        }
      }
    }
    hy_p = hy_c;
    hz_p = hz_c;
  }
}

// ---------------------------------------------------------------------------------------
// End of an iteration: electric sources on nodes outside the E kernel's domain, then the
// receiver samples that the next iteration starts from (fields_outputs.py:40-67, grid.py:
// 413-461), then the iteration counter advances.
struct RxParams {
  const int* coords;   // [nrx][3]
  float* out;          // [9][iterations][nrx]
  int nrx;
  int iterations;
  float dx, dy, dz;
  int nsrcOut;
  const Src* srcOut;
};

__global__ void end_of_step(const StepParams p, const RxParams r, int* d_it) {
  const int it = *d_it;
  if (threadIdx.x == 0) {
    for (int s = 0; s < r.nsrcOut; ++s) {
      const Src& q = r.srcOut[s];
      if (it < q.first || it > q.last) continue;
      const long long idx = (long long)q.i * p.sx + (long long)q.j * p.sy + q.k;
      float* E = p.E[q.comp];
      const uint32_t m = p.ID[q.comp * p.ncomp + idx];
      const float c4 = p.cE[5 * (long long)m + 4];
      const float w = q.w[it];
      float F = E[idx];
      if (q.kind == 0) F = __fsub_rn(F, __fmul_rn(__fmul_rn(__fmul_rn(c4, w), q.s0), q.s1));
      else if (q.kind == 1) F = __fsub_rn(F, __fmul_rn(__fmul_rn(c4, w), q.s0));
      else F = __fdiv_rn(-w, q.s0);
      E[idx] = F;
    }
  }
  __syncthreads();
  const int sample = it + 1;
  if (sample < r.iterations) {
    for (int n = threadIdx.x; n < r.nrx; n += blockDim.x) {
      const int x = r.coords[3 * n], y = r.coords[3 * n + 1], z = r.coords[3 * n + 2];
      const long long idx = (long long)x * p.sx + (long long)y * p.sy + z;
      float v[9];
      for (int c = 0; c < 3; ++c) v[c] = p.E[c][idx];
      for (int c = 0; c < 3; ++c) v[3 + c] = p.H[c][idx];
      const float* Hx = p.H[0];
      const float* Hy = p.H[1];
      const float* Hz = p.H[2];
      v[6] = (y == 0 || z == 0) ? 0.f :
          __fadd_rn(__fmul_rn(r.dy, __fsub_rn(Hy[idx - 1], Hy[idx])),
                    __fmul_rn(r.dz, __fsub_rn(Hz[idx], Hz[idx - p.sy])));
      v[7] = (x == 0 || z == 0) ? 0.f :
          __fadd_rn(__fmul_rn(r.dx, __fsub_rn(Hx[idx], Hx[idx - 1])),
                    __fmul_rn(r.dz, __fsub_rn(Hz[idx - p.sx], Hz[idx])));
      v[8] = (x == 0 || y == 0) ? 0.f :
          __fadd_rn(__fmul_rn(r.dx, __fsub_rn(Hx[idx - p.sy], Hx[idx])),
                    __fmul_rn(r.dy, __fsub_rn(Hy[idx], Hy[idx - p.sx])));
      for (int c = 0; c < 9; ++c)
        r.out[((long long)c * r.iterations + sample) * r.nrx + n] = v[c];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *d_it = it + 1;
}

// Snapshot: cell averages over a strided sub-volume (snapshots_ext.pyx:24-71).
struct SnapParams {
  int xs, ys, zs, sdx, sdy, sdz, snx, sny, snz;
  float* out;   // [6][snx][sny][snz]
};

__global__ void snapshot_store(const StepParams p, const SnapParams s) {
  const long long n = (long long)s.snx * s.sny * s.snz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int kk = (int)(q % s.snz);
    const int jj = (int)((q / s.snz) % s.sny);
    const int ii = (int)(q / ((long long)s.snz * s.sny));
    const long long base = (long long)(s.xs + ii * s.sdx) * p.sx +
                           (long long)(s.ys + jj * s.sdy) * p.sy + (s.zs + kk * s.sdz);
    const long long di = (long long)s.sdx * p.sx, dj = (long long)s.sdy * p.sy, dk = s.sdz;
    const float* Ex = p.E[0];
    const float* Ey = p.E[1];
    const float* Ez = p.E[2];
    const float* Hx = p.H[0];
    const float* Hy = p.H[1];
    const float* Hz = p.H[2];
    s.out[0 * n + q] = (Ex[base] + Ex[base + dj] + Ex[base + dk] + Ex[base + dj + dk]) / 4.f;
    s.out[1 * n + q] = (Ey[base] + Ey[base + di] + Ey[base + dk] + Ey[base + di + dk]) / 4.f;
    s.out[2 * n + q] = (Ez[base] + Ez[base + di] + Ez[base + dj] + Ez[base + di + dj]) / 4.f;
    s.out[3 * n + q] = (Hx[base] + Hx[base + di]) / 2.f;
    s.out[4 * n + q] = (Hy[base] + Hy[base + dj]) / 2.f;
    s.out[5 * n + q] = (Hz[base] + Hz[base + dk]) / 2.f;
  }
}

}  // namespace gbf
