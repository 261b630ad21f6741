// fdtd_kernels.cuh — fused Yee half-step kernels for sm_103a.
//
// One H kernel and one E kernel advance a whole time step. Each touches every field value,
// material ID and PML/dispersive state word it needs once per half-step:
//
//   H half-step  gprMax/fields_updates_ext.pyx:352-412 (update_magnetic), then the six
//                pml_updates_magnetic_*_ext.pyx slab corrections in slab order, then the
//                magnetic-dipole sources (model_build_run.py:434-442)
//   E half-step  update_electric (:30-110) or update_electric_dispersive_*_A (:113-297), the six
//                pml_updates_electric_*_ext.pyx corrections, voltage sources and Hertzian
//                dipoles, then the dispersive part B (:183-349) with the final E
//                (model_build_run.py:444-470)
//
// Every term is the reference's arithmetic in the reference's order (main update; slab
// corrections in the order x0, y0, z0, xmax, ymax, zmax; sources; part B). Only the schedule
// differs: the thread that owns a node applies all of them in registers. Built without
// floating-point contraction, the results are bit-identical to the reference's CPU kernels
// compiled the same way.
//
// Thread mapping: a block covers 32 consecutive k (one warp per row) by kBY rows j and walks a
// chunk of x planes, carrying the neighbouring plane of the other field in registers. Slab
// membership along y and z is fixed per thread and along x per plane, so nodes outside the
// PML take a path without any PML work. The coefficient tables are staged in shared memory
// when they fit (the reference keeps them in __constant__ memory, model_build_run.py:512-519).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbf {

constexpr int kBX = 32;   // k extent of a block (one warp)
constexpr int kBY = 8;    // j extent of a block
constexpr int kMaxPoles = 4;
constexpr int kSmemCoefMax = 2048;   // materials staged in shared memory

// PML kinds: formulation x order (pml.py:156-159 and len(G.cfs))
enum PmlKind : int { PML_NONE = 0, PML_HORI1 = 1, PML_HORI2 = 2, PML_MRI1 = 3, PML_MRI2 = 4 };

// Slab positions in application order: x0, y0, z0, xmax, ymax, zmax (axis = s % 3).
struct Slab {
  int T;            // thickness in cells, 0 = absent
  float d;          // cell size along the axis (fp32, the reference kernels' `float d`)
  long long ocount; // Phi elements per CFS order
  float* phiE1;     // Phi arrays [order][...] of the first/second tangential E component
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
  const uint32_t* ID[6];  // per component [ncomp]
  int ncomp;              // nodes per component (< 2^31)
  int nx, ny, nz;
  int sy, sx;             // strides: j -> nz+1, i -> (ny+1)(nz+1)
  const float4* cE4;      // [nmat] CA, CBx, CBy, CBz
  const float* cEs;       // [nmat] srce
  const float4* cH4;      // [nmat] DA, DBx, DBy, DBz
  const float* cHs;       // [nmat] srcm
  const float2* cD;       // [nmat][3P]
  int nmat;
  int smem;               // 1: tables staged in shared memory
  float2* T;              // [3][P][ncomp]
  int P;
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
// RA01, IRA, RC0 ... are recomputed from the stored rows exactly as the reference does.
template <int PK>
__device__ __forceinline__ float pml_term(float dF, float* phi, long long pidx, long long ocount,
                                          const float* __restrict__ R, int T, int p) {
  constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  const float RA0 = __ldg(R + (0 * order + 0) * T + p);
  const float RB0 = __ldg(R + (1 * order + 0) * T + p);
  const float RE0 = __ldg(R + (2 * order + 0) * T + p);
  const float RF0 = __ldg(R + (3 * order + 0) * T + p);
  const float ph0 = phi[pidx];
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
    const float ph1 = phi[pidx + ocount];
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
    const float ph1 = phi[pidx + ocount];
    const float Psi = RB0 * ph0 + RB1 * ph1;
    const float X = IRA1 * dF - IRA * Psi;
    phi[pidx + ocount] = RE1 * ph1 + RC1 * (dF - Psi);
    phi[pidx] = RE0 * ph0 + RC0 * (dF - Psi);
    return X;
  }
}

// Phi index of node (i, j, k) at profile index p (layouts: x [p][j][k], y [i][p][k], z [i][j][p]).
template <int AXIS>
__device__ __forceinline__ long long phi_index(int i, int j, int k, int p, int T, int ny, int nz) {
  if (AXIS == 0) return ((long long)p * ny + j) * nz + k;
  if (AXIS == 1) return ((long long)i * T + p) * nz + k;
  return ((long long)i * ny + j) * T + p;
}

// Slab membership and profile index of coordinate c along a slab's axis.
// E ranges: minus c in [1, T] (p = T - c), plus c in [n - T, n - 1] (p = c - (n - T)).
// H ranges: minus c in [0, T - 1] (p = T - 1 - c), plus as E.
template <bool ELECTRIC>
__device__ __forceinline__ int slab_p(int c, int T, int n, bool minus) {
  if (T == 0) return -1;
  if (minus) {
    if (ELECTRIC) return (c >= 1 && c <= T) ? T - c : -1;
    return (c < T) ? T - 1 - c : -1;
  }
  return (c >= n - T && c < n) ? c - (n - T) : -1;
}

// Stage the coefficient tables in shared memory (when they fit).
__device__ __forceinline__ void stage_tables(const StepParams& p, bool electric, float4* s4,
                                             float* ss, float2* sd) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nt = blockDim.x * blockDim.y;
  const float4* g4 = electric ? p.cE4 : p.cH4;
  const float* gs = electric ? p.cEs : p.cHs;
  for (int m = tid; m < p.nmat; m += nt) {
    s4[m] = __ldg(g4 + m);
    ss[m] = __ldg(gs + m);
  }
  if (electric && sd) {
    const int nd = p.nmat * 3 * p.P;
    for (int q = tid; q < nd; q += nt) sd[q] = __ldg(p.cD + q);
  }
}

// ---------------------------------------------------------------------------------------
// H half-step. Domain: i in [0, nx], j in [0, ny], k in [0, nz].
template <int PK>
__global__ void __launch_bounds__(kBX * kBY, 3)
h_half_step(const __grid_constant__ StepParams p) {
  extern __shared__ float4 smem_h[];
  float4* s4 = smem_h;
  float* ss = reinterpret_cast<float*>(s4 + (p.smem ? p.nmat : 0));
  if (p.smem) {
    stage_tables(p, false, s4, ss, nullptr);
    __syncthreads();
  }
  const float4* C4 = p.smem ? s4 : p.cH4;
  const float* Cs = p.smem ? ss : p.cHs;
  const int k = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (k > p.nz || j > p.ny) return;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int i0 = blockIdx.z * p.chunk;
  const int i1 = min(i0 + p.chunk, nx + 1);
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  float* __restrict__ Hx = p.H[0];
  float* __restrict__ Hy = p.H[1];
  float* __restrict__ Hz = p.H[2];
  const bool jin = j < ny, kin = k < nz;

  // PML membership fixed for this thread (y and z); every H slab range needs i < nx, j < ny
  // and k < nz, so these also apply only on planes i < nx (checked per plane below)
  int py0 = -1, pymax = -1, pz0 = -1, pzmax = -1;
  if (PK != PML_NONE && jin && kin) {
    py0 = slab_p<false>(j, p.slab[1].T, ny, true);
    pymax = slab_p<false>(j, p.slab[4].T, ny, false);
    pz0 = slab_p<false>(k, p.slab[2].T, nz, true);
    pzmax = slab_p<false>(k, p.slab[5].T, nz, false);
  }
  // magnetic sources owned by this thread's (j, k) column
  bool colsrc = false;
  for (int s = 0; s < p.nsrcH; ++s) {
    const Src& q = p.srcH[s];
    if (q.j == j && q.k == k && q.i >= i0 && q.i < i1) colsrc = true;
  }
  const int it = colsrc ? *p.d_it : 0;

  int idx = i0 * p.sx + j * p.sy + k;
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
    // every load of the plane is issued before any store, so they are all in flight together
    const uint32_t mx = __ldg(p.ID[3] + idx);
    const uint32_t my = __ldg(p.ID[4] + idx);
    const uint32_t mz = __ldg(p.ID[5] + idx);
    const float hx0 = Hx[idx], hy0 = Hy[idx], hz0 = Hz[idx];
    const float dEz_y = ez_j - ez_c;   // Hx main and y-slab
    const float dEy_z = ey_k - ey_c;   // Hx main and z-slab
    const float dEx_z = ex_k - ex_c;   // Hy main and z-slab
    const float dEz_x = ez_n - ez_c;   // Hy main and x-slab
    const float dEy_x = ey_n - ey_c;   // Hz main and x-slab
    const float dEx_y = ex_j - ex_c;   // Hz main and y-slab
    int px0 = -1, pxmax = -1;
    const bool iin = i < nx;
    if (PK != PML_NONE && iin && jin && kin) {
      px0 = slab_p<false>(i, p.slab[0].T, nx, true);
      pxmax = slab_p<false>(i, p.slab[3].T, nx, false);
    }
    const bool src = colsrc;

    // ---- Hx: main i in [1,nx], j in [0,ny), k in [0,nz); PML y-slabs (-, Phi1), z-slabs (+, Phi1)
    {
      const bool mainu = (i >= 1) && jin && kin;
      // slab corrections cover i < nx only (the main update also covers i = nx)
      const bool pml = PK != PML_NONE && iin &&
                       (py0 >= 0 || pymax >= 0 || pz0 >= 0 || pzmax >= 0);
      if (mainu || pml || src) {
        const uint32_t m = mx;
        float F = hx0;
        if (mainu) {
          const float4 c = C4[m];
          F = c.x * F - c.z * dEz_y + c.w * dEy_z;
        }
        if (PK != PML_NONE && pml) {
          const float c4 = Cs[m];
          if (py0 >= 0) {
            const Slab& sl = p.slab[1];
            const float X = pml_term<PK>(dEz_y / sl.d, sl.phiH1, phi_index<1>(i, j, k, py0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, py0);
            F = F - c4 * X;
          }
          if (pz0 >= 0) {
            const Slab& sl = p.slab[2];
            const float X = pml_term<PK>(dEy_z / sl.d, sl.phiH1, phi_index<2>(i, j, k, pz0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pz0);
            F = F + c4 * X;
          }
          if (pymax >= 0) {
            const Slab& sl = p.slab[4];
            const float X = pml_term<PK>(dEz_y / sl.d, sl.phiH1, phi_index<1>(i, j, k, pymax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pymax);
            F = F - c4 * X;
          }
          if (pzmax >= 0) {
            const Slab& sl = p.slab[5];
            const float X = pml_term<PK>(dEy_z / sl.d, sl.phiH1, phi_index<2>(i, j, k, pzmax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pzmax);
            F = F + c4 * X;
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 3 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(Cs[m], __ldg(q.w + it)), q.s0));
          }
        }
        Hx[idx] = F;
      }
    }
    // ---- Hy: main i in [0,nx), j in [1,ny], k in [0,nz); PML x-slabs (+, Phi1), z-slabs (-, Phi2)
    {
      const bool mainu = iin && (j >= 1) && kin;
      const bool pml = PK != PML_NONE && iin && (px0 >= 0 || pxmax >= 0 || pz0 >= 0 || pzmax >= 0);
      if (mainu || pml || src) {
        const uint32_t m = my;
        float F = hy0;
        if (mainu) {
          const float4 c = C4[m];
          F = c.x * F - c.w * dEx_z + c.y * dEz_x;
        }
        if (PK != PML_NONE && pml) {
          const float c4 = Cs[m];
          if (px0 >= 0) {
            const Slab& sl = p.slab[0];
            const float X = pml_term<PK>(dEz_x / sl.d, sl.phiH1, phi_index<0>(i, j, k, px0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, px0);
            F = F + c4 * X;
          }
          if (pz0 >= 0) {
            const Slab& sl = p.slab[2];
            const float X = pml_term<PK>(dEx_z / sl.d, sl.phiH2, phi_index<2>(i, j, k, pz0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pz0);
            F = F - c4 * X;
          }
          if (pxmax >= 0) {
            const Slab& sl = p.slab[3];
            const float X = pml_term<PK>(dEz_x / sl.d, sl.phiH1, phi_index<0>(i, j, k, pxmax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pxmax);
            F = F + c4 * X;
          }
          if (pzmax >= 0) {
            const Slab& sl = p.slab[5];
            const float X = pml_term<PK>(dEx_z / sl.d, sl.phiH2, phi_index<2>(i, j, k, pzmax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pzmax);
            F = F - c4 * X;
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 4 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(Cs[m], __ldg(q.w + it)), q.s0));
          }
        }
        Hy[idx] = F;
      }
    }
    // ---- Hz: main i in [0,nx), j in [0,ny), k in [1,nz]; PML x-slabs (-, Phi2), y-slabs (+, Phi2)
    {
      const bool mainu = iin && jin && (k >= 1);
      const bool pml = PK != PML_NONE && iin && (px0 >= 0 || pxmax >= 0 || py0 >= 0 || pymax >= 0);
      if (mainu || pml || src) {
        const uint32_t m = mz;
        float F = hz0;
        if (mainu) {
          const float4 c = C4[m];
          F = c.x * F - c.y * dEy_x + c.z * dEx_y;
        }
        if (PK != PML_NONE && pml) {
          const float c4 = Cs[m];
          if (px0 >= 0) {
            const Slab& sl = p.slab[0];
            const float X = pml_term<PK>(dEy_x / sl.d, sl.phiH2, phi_index<0>(i, j, k, px0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, px0);
            F = F - c4 * X;
          }
          if (py0 >= 0) {
            const Slab& sl = p.slab[1];
            const float X = pml_term<PK>(dEx_y / sl.d, sl.phiH2, phi_index<1>(i, j, k, py0, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, py0);
            F = F + c4 * X;
          }
          if (pxmax >= 0) {
            const Slab& sl = p.slab[3];
            const float X = pml_term<PK>(dEy_x / sl.d, sl.phiH2, phi_index<0>(i, j, k, pxmax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pxmax);
            F = F - c4 * X;
          }
          if (pymax >= 0) {
            const Slab& sl = p.slab[4];
            const float X = pml_term<PK>(dEx_y / sl.d, sl.phiH2, phi_index<1>(i, j, k, pymax, sl.T, ny, nz), sl.ocount, sl.hR, sl.T, pymax);
            F = F + c4 * X;
          }
        }
        if (src) {
          for (int s = 0; s < p.nsrcH; ++s) {
            const Src& q = p.srcH[s];
            if (q.comp == 5 && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
              F = __fsub_rn(F, __fmul_rn(__fmul_rn(Cs[m], __ldg(q.w + it)), q.s0));
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

// One slab's correction of one E component (compile-time slab position S and component C).
// Table per slab axis: x-slab Ey (Phi1, dHz/dx, -), Ez (Phi2, dHy/dx, +); y-slab Ex (Phi1,
// dHz/dy, +), Ez (Phi2, dHx/dy, -); z-slab Ex (Phi1, dHy/dz, -), Ey (Phi2, dHx/dz, +).
template <int PK, int S, int C>
__device__ __forceinline__ float e_slab(float F, float c4, int pp, int i, int j, int k,
                                        float dA, float dB, const StepParams& p) {
  constexpr int AX = S % 3;
  const Slab& sl = p.slab[S];
  constexpr bool first = (AX == 0) ? (C == 1) : (C == 0);
  constexpr float sgn = (AX == 0) ? (C == 1 ? -1.f : 1.f) : (AX == 1) ? (C == 0 ? 1.f : -1.f)
                                                                      : (C == 0 ? -1.f : 1.f);
  const float dF = first ? dA : dB;
  const float X = pml_term<PK>(dF / sl.d, first ? sl.phiE1 : sl.phiE2,
                               phi_index<AX>(i, j, k, pp, sl.T, p.ny, p.nz), sl.ocount, sl.eR,
                               sl.T, pp);
  return sgn > 0.f ? F + c4 * X : F - c4 * X;
}

// E half-step. Domain: i in [0, nx), j in [0, ny), k in [0, nz). NP = dispersive poles.
template <int PK, int NP>
__global__ void __launch_bounds__(kBX * kBY, 3)
e_half_step(const __grid_constant__ StepParams p) {
  extern __shared__ float4 smem_e[];
  float4* s4 = smem_e;
  float* ss = reinterpret_cast<float*>(s4 + (p.smem ? p.nmat : 0));
  float2* sd = reinterpret_cast<float2*>(ss + (p.smem ? ((p.nmat + 1) & ~1) : 0));
  if (p.smem) {
    stage_tables(p, true, s4, ss, NP > 0 ? sd : nullptr);
    __syncthreads();
  }
  const float4* C4 = p.smem ? s4 : p.cE4;
  const float* Cs = p.smem ? ss : p.cEs;
  const float2* CD = (p.smem && NP > 0) ? sd : p.cD;
  const int k = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int i0 = blockIdx.z * p.chunk;
  const int i1 = min(i0 + p.chunk, nx);
  const float* __restrict__ Hx = p.H[0];
  const float* __restrict__ Hy = p.H[1];
  const float* __restrict__ Hz = p.H[2];

  int py0 = -1, pymax = -1, pz0 = -1, pzmax = -1;
  if (PK != PML_NONE) {
    py0 = slab_p<true>(j, p.slab[1].T, ny, true);
    pymax = slab_p<true>(j, p.slab[4].T, ny, false);
    pz0 = slab_p<true>(k, p.slab[2].T, nz, true);
    pzmax = slab_p<true>(k, p.slab[5].T, nz, false);
  }
  bool colsrc = false;
  for (int s = 0; s < p.nsrcE; ++s) {
    const Src& q = p.srcE[s];
    if (q.j == j && q.k == k && q.i >= i0 && q.i < i1) colsrc = true;
  }
  const int it = colsrc ? *p.d_it : 0;

  int idx = i0 * p.sx + j * p.sy + k;
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
    int px0 = -1, pxmax = -1;
    if (PK != PML_NONE) {
      px0 = slab_p<true>(i, p.slab[0].T, nx, true);
      pxmax = slab_p<true>(i, p.slab[3].T, nx, false);
    }
    const bool src = colsrc;
    // every load of the plane is issued before any store, so they are all in flight together
    uint32_t mm[3];
    float eold[3];
    float2 tt[3][NP > 0 ? NP : 1];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      mm[comp] = __ldg(p.ID[comp] + idx);
      eold[comp] = p.E[comp][idx];
#pragma unroll
      for (int q = 0; q < NP; ++q)
        tt[comp][q] = p.T[(comp * NP + q) * (long long)p.ncomp + idx];
    }

#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      bool mainu, pml;
      if (comp == 0) {
        mainu = (j >= 1) && (k >= 1);
        pml = py0 >= 0 || pymax >= 0 || pz0 >= 0 || pzmax >= 0;
      } else if (comp == 1) {
        mainu = (i >= 1) && (k >= 1);
        pml = px0 >= 0 || pxmax >= 0 || pz0 >= 0 || pzmax >= 0;
      } else {
        mainu = (i >= 1) && (j >= 1);
        pml = px0 >= 0 || pxmax >= 0 || py0 >= 0 || pymax >= 0;
      }
      if (PK == PML_NONE) pml = false;
      if (!(mainu || pml || src)) continue;
      float* __restrict__ E = p.E[comp];
      const uint32_t m = mm[comp];
      const float Eold = eold[comp];
      float F = Eold;
      float2 TA[NP > 0 ? NP : 1];
      if (mainu) {
        // curl terms in the reference's order: CA*E + CB1*d1 - CB2*d2
        const float4 c = C4[m];
        float t1, t2;
        if (comp == 0) { t1 = c.z * dHz_y; t2 = c.w * dHy_z; }
        else if (comp == 1) { t1 = c.w * dHx_z; t2 = c.y * dHz_x; }
        else { t1 = c.y * dHy_x; t2 = c.z * dHx_y; }
        if (NP == 0) {
          F = c.x * Eold + t1 - t2;
        } else {
          float phi = 0.f;
          const float2* cd = CD + m * 3 * NP;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const float2 Tq = tt[comp][q];
            const float2 a = cd[3 * q + 0];
            const float2 b = cd[3 * q + 1];
            const float2 z = cd[3 * q + 2];
            phi = phi + a.x * Tq.x;
            TA[q].x = (b.x * Tq.x - b.y * Tq.y) + z.x * Eold;
            TA[q].y = (b.x * Tq.y + b.y * Tq.x) + z.y * Eold;
          }
          F = c.x * Eold + t1 - t2 - Cs[m] * phi;
        }
      }
      if (PK != PML_NONE && pml) {
        const float c4 = Cs[m];
        // slab order x0, y0, z0, xmax, ymax, zmax; a component is tangential to two axes
        if (comp == 0) {
          if (py0 >= 0) F = e_slab<PK, 1, 0>(F, c4, py0, i, j, k, dHz_y, dHx_y, p);
          if (pz0 >= 0) F = e_slab<PK, 2, 0>(F, c4, pz0, i, j, k, dHy_z, dHx_z, p);
          if (pymax >= 0) F = e_slab<PK, 4, 0>(F, c4, pymax, i, j, k, dHz_y, dHx_y, p);
          if (pzmax >= 0) F = e_slab<PK, 5, 0>(F, c4, pzmax, i, j, k, dHy_z, dHx_z, p);
        } else if (comp == 1) {
          if (px0 >= 0) F = e_slab<PK, 0, 1>(F, c4, px0, i, j, k, dHz_x, dHy_x, p);
          if (pz0 >= 0) F = e_slab<PK, 2, 1>(F, c4, pz0, i, j, k, dHy_z, dHx_z, p);
          if (pxmax >= 0) F = e_slab<PK, 3, 1>(F, c4, pxmax, i, j, k, dHz_x, dHy_x, p);
          if (pzmax >= 0) F = e_slab<PK, 5, 1>(F, c4, pzmax, i, j, k, dHy_z, dHx_z, p);
        } else {
          if (px0 >= 0) F = e_slab<PK, 0, 2>(F, c4, px0, i, j, k, dHz_x, dHy_x, p);
          if (py0 >= 0) F = e_slab<PK, 1, 2>(F, c4, py0, i, j, k, dHz_y, dHx_y, p);
          if (pxmax >= 0) F = e_slab<PK, 3, 2>(F, c4, pxmax, i, j, k, dHz_x, dHy_x, p);
          if (pymax >= 0) F = e_slab<PK, 4, 2>(F, c4, pymax, i, j, k, dHz_y, dHx_y, p);
        }
      }
      if (src) F = apply_e_sources(F, comp, i, j, k, it, Cs[m], p);
      E[idx] = F;
      if (NP > 0 && mainu) {
        const float2* cd = CD + m * 3 * NP;
        float2* Tc = p.T + (comp * NP) * (long long)p.ncomp + idx;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float2 z = cd[3 * q + 2];
          float2 o;
          o.x = TA[q].x - z.x * F;
          o.y = TA[q].y - z.y * F;
          Tc[q * (long long)p.ncomp] = o;
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

__global__ void end_of_step(const __grid_constant__ StepParams p, const __grid_constant__ RxParams r, int* d_it) {
  const int it = *d_it;
  if (threadIdx.x == 0) {
    for (int s = 0; s < r.nsrcOut; ++s) {
      const Src& q = r.srcOut[s];
      if (it < q.first || it > q.last) continue;
      const long long idx = (long long)q.i * p.sx + (long long)q.j * p.sy + q.k;
      float* E = p.E[q.comp];
      const uint32_t m = p.ID[q.comp][idx];
      const float c4 = p.cEs[m];
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

__global__ void snapshot_store(const __grid_constant__ StepParams p, const SnapParams s) {
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
