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
// Thread mapping: a persistent grid sweeps the flattened node index in order (consecutive
// threads on consecutive nodes), one node per thread per pass. Nodes outside the PML box skip
// all PML work. The coefficient tables are staged in shared memory when they fit (the reference
// keeps them in __constant__ memory, model_build_run.py:512-519).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbf {

constexpr int kThreads = 256;   // threads per block of the half-step kernels
constexpr int kSrcInline = 8;   // sources whose node index travels in the kernel parameters
constexpr int kPackBits = 10;   // bits per material ID in a packed word (IDs < 1024)
constexpr uint32_t kPackMask = (1u << kPackBits) - 1u;
constexpr uint32_t kDispersiveBit = 1u << 30;
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

struct StepParams;
typedef void (*HKernFn)(StepParams);
typedef void (*EKernFn)(StepParams);
// per-kind kernel tables (kernels_inst.cu, one object per PML kind)
void kernels_pk0(int np, int idp, HKernFn* h, EKernFn* e);
void kernels_pk1(int np, int idp, HKernFn* h, EKernFn* e);
void kernels_pk2(int np, int idp, HKernFn* h, EKernFn* e);
void kernels_pk3(int np, int idp, HKernFn* h, EKernFn* e);
void kernels_pk4(int np, int idp, HKernFn* h, EKernFn* e);

struct Src {
  int kind, comp, i, j, k, first, last, pad;
  float s0, s1;
  const float* w;   // this source's waveform table [iterations]
};

struct StepParams {
  float* E[3];
  float* H[3];
  const uint32_t* ID[6];  // per component [ncomp]
  const uint32_t* PE;     // packed E IDs per node: x | y << 10 | z << 20 | dispersive << 30
  const uint32_t* PH;     // packed H IDs per node: x | y << 10 | z << 20
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
  int srcqE[kSrcInline];  // flat node index of the first sources (lets a node test itself cheaply)
  int srcqH[kSrcInline];
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
// Flat persistent sweep: threads take consecutive nodes of the flattened (i, j, k) index, and a
// grid of a few blocks per SM strides through the whole array in order, so every array is
// streamed front to back by the whole GPU at once (DRAM-page friendly for the ~20 concurrent
// streams of a half-step). Neighbours along j, k (and x) are re-read from L1/L2.
// The node index is advanced incrementally: the stride splits into whole planes, rows and nodes.
struct FlatWalk {
  int i, j, k, si, sj, sk, rows;
  __device__ __forceinline__ FlatWalk(long long q, long long stride, int sx, int sy, int nrows) {
    rows = nrows;
    i = (int)(q / sx);
    int r = (int)(q - (long long)i * sx);
    j = r / sy;
    k = r - j * sy;
    si = (int)(stride / sx);
    r = (int)(stride - (long long)si * sx);
    sj = r / sy;
    sk = r - sj * sy;
  }
  __device__ __forceinline__ void advance(int sy) {
    k += sk;
    if (k >= sy) { k -= sy; ++j; }
    j += sj;
    if (j >= rows) { j -= rows; ++i; }
    i += si;
  }
};

// One slab's correction of one H component (compile-time slab position S, component C).
// Table per slab axis: x-slab Hy (Phi1, dEz/dx, +), Hz (Phi2, dEy/dx, -); y-slab Hx (Phi1,
// dEz/dy, -), Hz (Phi2, dEx/dy, +); z-slab Hx (Phi1, dEy/dz, +), Hy (Phi2, dEx/dz, -).
template <int PK, int S, int C>
__device__ __forceinline__ float h_slab(float F, float c4, int pp, int i, int j, int k,
                                        float dA, float dB, const StepParams& p) {
  constexpr int AX = S % 3;
  const Slab& sl = p.slab[S];
  constexpr bool first = (AX == 0) ? (C == 1) : (C == 0);
  constexpr float sgn = (AX == 0) ? (C == 1 ? 1.f : -1.f) : (AX == 1) ? (C == 0 ? -1.f : 1.f)
                                                                      : (C == 0 ? 1.f : -1.f);
  const float dF = first ? dA : dB;
  const float X = pml_term<PK>(dF / sl.d, first ? sl.phiH1 : sl.phiH2,
                               phi_index<AX>(i, j, k, pp, sl.T, p.ny, p.nz), sl.ocount, sl.hR,
                               sl.T, pp);
  return sgn > 0.f ? F + c4 * X : F - c4 * X;
}

// Magnetic sources at one node/component (sources.py:202-232, numpy-2 fp32 order).
__device__ __forceinline__ float apply_h_sources(float F, int comp, int i, int j, int k, int it,
                                                 float c4, const StepParams& p) {
  for (int s = 0; s < p.nsrcH; ++s) {
    const Src& q = p.srcH[s];
    if (q.comp == comp && q.i == i && q.j == j && q.k == k && it >= q.first && it <= q.last)
      F = __fsub_rn(F, __fmul_rn(__fmul_rn(c4, __ldg(q.w + it)), q.s0));
  }
  return F;
}

// Does any source sit on flat node `idx`? The first kSrcInline sources are tested from the
// kernel parameters; further ones from their list.
__device__ __forceinline__ bool node_has_source(int idx, int n, const int* inl, const Src* list,
                                                int sx, int sy) {
  bool hit = false;
  const int m = n < kSrcInline ? n : kSrcInline;
  for (int s = 0; s < m; ++s) hit |= (inl[s] == idx);
  for (int s = kSrcInline; s < n; ++s) {
    const Src& q = list[s];
    hit |= (q.i * sx + q.j * sy + q.k == idx);
  }
  return hit;
}

// H update of one node: main update (update_magnetic), slab corrections in slab order, sources.
// px0/pxmax/py0/pymax are the node's x and y slab profile indices (-1 outside).
template <int PK>
__device__ __forceinline__ void h_node(const StepParams& p, const float4* C4, const float* Cs,
                                       int i, int j, int k, bool src, int it, int px0, int pxmax,
                                       int py0, int pymax, int pz0, int pzmax, float dEz_y,
                                       float dEy_z, float dEx_z,
                                       float dEz_x, float dEy_x, float dEx_y, uint32_t mx,
                                       uint32_t my, uint32_t mz, float& hx, float& hy, float& hz) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const bool iin = i < nx, jin = j < ny, kin = k < nz;
  // every H slab range needs i < nx, j < ny and k < nz
  const bool inpml = PK != PML_NONE && iin && jin && kin;
  // Hx: main i in [1,nx], j in [0,ny), k in [0,nz); slabs y0, z0, ymax, zmax
  {
    const bool mainu = (i >= 1) && jin && kin;
    const bool pml = inpml && (py0 >= 0 || pymax >= 0 || pz0 >= 0 || pzmax >= 0);
    if (mainu || pml || src) {
      float F = hx;
      if (mainu) {
        const float4 c = C4[mx];
        F = c.x * F - c.z * dEz_y + c.w * dEy_z;
      }
      if (PK != PML_NONE && pml) {
        const float c4 = Cs[mx];
        if (py0 >= 0) F = h_slab<PK, 1, 0>(F, c4, py0, i, j, k, dEz_y, dEx_y, p);
        if (pz0 >= 0) F = h_slab<PK, 2, 0>(F, c4, pz0, i, j, k, dEy_z, dEx_z, p);
        if (pymax >= 0) F = h_slab<PK, 4, 0>(F, c4, pymax, i, j, k, dEz_y, dEx_y, p);
        if (pzmax >= 0) F = h_slab<PK, 5, 0>(F, c4, pzmax, i, j, k, dEy_z, dEx_z, p);
      }
      if (src) F = apply_h_sources(F, 3, i, j, k, it, Cs[mx], p);
      hx = F;
    }
  }
  // Hy: main i in [0,nx), j in [1,ny], k in [0,nz); slabs x0, z0, xmax, zmax
  {
    const bool mainu = iin && (j >= 1) && kin;
    const bool pml = inpml && (px0 >= 0 || pxmax >= 0 || pz0 >= 0 || pzmax >= 0);
    if (mainu || pml || src) {
      float F = hy;
      if (mainu) {
        const float4 c = C4[my];
        F = c.x * F - c.w * dEx_z + c.y * dEz_x;
      }
      if (PK != PML_NONE && pml) {
        const float c4 = Cs[my];
        if (px0 >= 0) F = h_slab<PK, 0, 1>(F, c4, px0, i, j, k, dEz_x, dEy_x, p);
        if (pz0 >= 0) F = h_slab<PK, 2, 1>(F, c4, pz0, i, j, k, dEy_z, dEx_z, p);
        if (pxmax >= 0) F = h_slab<PK, 3, 1>(F, c4, pxmax, i, j, k, dEz_x, dEy_x, p);
        if (pzmax >= 0) F = h_slab<PK, 5, 1>(F, c4, pzmax, i, j, k, dEy_z, dEx_z, p);
      }
      if (src) F = apply_h_sources(F, 4, i, j, k, it, Cs[my], p);
      hy = F;
    }
  }
  // Hz: main i in [0,nx), j in [0,ny), k in [1,nz]; slabs x0, y0, xmax, ymax
  {
    const bool mainu = iin && jin && (k >= 1);
    const bool pml = inpml && (px0 >= 0 || pxmax >= 0 || py0 >= 0 || pymax >= 0);
    if (mainu || pml || src) {
      float F = hz;
      if (mainu) {
        const float4 c = C4[mz];
        F = c.x * F - c.y * dEy_x + c.z * dEx_y;
      }
      if (PK != PML_NONE && pml) {
        const float c4 = Cs[mz];
        if (px0 >= 0) F = h_slab<PK, 0, 2>(F, c4, px0, i, j, k, dEz_x, dEy_x, p);
        if (py0 >= 0) F = h_slab<PK, 1, 2>(F, c4, py0, i, j, k, dEz_y, dEx_y, p);
        if (pxmax >= 0) F = h_slab<PK, 3, 2>(F, c4, pxmax, i, j, k, dEz_x, dEy_x, p);
        if (pymax >= 0) F = h_slab<PK, 4, 2>(F, c4, pymax, i, j, k, dEz_y, dEx_y, p);
      }
      if (src) F = apply_h_sources(F, 5, i, j, k, it, Cs[mz], p);
      hz = F;
    }
  }
}

// H half-step. Domain: i in [0, nx], j in [0, ny], k in [0, nz] (every node of the arrays).
template <int PK, int IDP>
__global__ void __launch_bounds__(kThreads, 5)
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
  const int nx = p.nx, ny = p.ny, nz = p.nz, sx = p.sx, sy = p.sy;
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  float* __restrict__ Hx = p.H[0];
  float* __restrict__ Hy = p.H[1];
  float* __restrict__ Hz = p.H[2];
  const long long total = (long long)(nx + 1) * sx;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  FlatWalk w(q, stride, sx, sy, ny + 1);
  // interior box: nodes outside every H slab range (minus [0,T-1], plus [n-T, n-1])
  const int xlo = p.slab[0].T, xhi = nx - p.slab[3].T;
  const int ylo = p.slab[1].T, yhi = ny - p.slab[4].T;
  const int zlo = p.slab[2].T, zhi = nz - p.slab[5].T;
  int it = 0;
  if (p.nsrcH) it = *p.d_it;
  for (; q < total; q += stride, w.advance(sy)) {
    const int idx = (int)q;
    const int i = w.i, j = w.j, k = w.k;
    const bool iin = i < nx, jin = j < ny, kin = k < nz;
    // issue every load of the node before any store
    const float ex_c = __ldg(Ex + idx), ey_c = __ldg(Ey + idx), ez_c = __ldg(Ez + idx);
    const float ex_j = jin ? __ldg(Ex + idx + sy) : 0.f;
    const float ez_j = jin ? __ldg(Ez + idx + sy) : 0.f;
    const float ex_k = kin ? __ldg(Ex + idx + 1) : 0.f;
    const float ey_k = kin ? __ldg(Ey + idx + 1) : 0.f;
    const float ey_n = iin ? __ldg(Ey + idx + sx) : 0.f;
    const float ez_n = iin ? __ldg(Ez + idx + sx) : 0.f;
    uint32_t mx, my, mz;
    if (IDP == 1) {
      const uint32_t w = __ldg(p.PH + idx);
      mx = w & kPackMask;
      my = (w >> kPackBits) & kPackMask;
      mz = (w >> (2 * kPackBits)) & kPackMask;
    } else {
      mx = __ldg(p.ID[3] + idx);
      my = __ldg(p.ID[4] + idx);
      mz = __ldg(p.ID[5] + idx);
    }
    float hx = Hx[idx], hy = Hy[idx], hz = Hz[idx];
    int px0 = -1, pxmax = -1, py0 = -1, pymax = -1, pz0 = -1, pzmax = -1;
    if (PK != PML_NONE && !(i >= xlo && i < xhi && j >= ylo && j < yhi && k >= zlo && k < zhi)) {
      px0 = slab_p<false>(i, p.slab[0].T, nx, true);
      pxmax = slab_p<false>(i, p.slab[3].T, nx, false);
      py0 = slab_p<false>(j, p.slab[1].T, ny, true);
      pymax = slab_p<false>(j, p.slab[4].T, ny, false);
      pz0 = slab_p<false>(k, p.slab[2].T, nz, true);
      pzmax = slab_p<false>(k, p.slab[5].T, nz, false);
    }
    const bool src = p.nsrcH && node_has_source(idx, p.nsrcH, p.srcqH, p.srcH, sx, sy);
    h_node<PK>(p, C4, Cs, i, j, k, src, it, px0, pxmax, py0, pymax, pz0, pzmax, ez_j - ez_c, ey_k - ey_c,
               ex_k - ex_c, ez_n - ez_c, ey_n - ey_c, ex_j - ex_c, mx, my, mz, hx, hy, hz);
    Hx[idx] = hx;
    Hy[idx] = hy;
    Hz[idx] = hz;
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

// E update of one node for all three components: main update (update_electric, or part A of
// the dispersive update), slab corrections in slab order, sources, dispersive part B.
template <int PK, int NP>
__device__ __forceinline__ void e_node(const StepParams& p, const float4* C4, const float* Cs,
                                       const float2* CD, int i, int j, int k, bool src, int it,
                                       int px0, int pxmax, int py0, int pymax, int pz0,
                                       int pzmax, float dHz_y,
                                       float dHy_z, float dHx_z, float dHz_x, float dHy_x,
                                       float dHx_y, const uint32_t* m, float* e, float2 (*t)[NP > 0 ? NP : 1]) {
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
    const uint32_t mm = m[comp];
    const float Eold = e[comp];
    float F = Eold;
    float2 TA[NP > 0 ? NP : 1];
    if (mainu) {
      // curl terms in the reference's order: CA*E + CB1*d1 - CB2*d2
      const float4 c = C4[mm];
      float t1, t2;
      if (comp == 0) { t1 = c.z * dHz_y; t2 = c.w * dHy_z; }
      else if (comp == 1) { t1 = c.w * dHx_z; t2 = c.y * dHz_x; }
      else { t1 = c.y * dHy_x; t2 = c.z * dHx_y; }
      if (NP == 0) {
        F = c.x * Eold + t1 - t2;
      } else {
        float phi = 0.f;
        const float2* cd = CD + mm * 3 * NP;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float2 Tq = t[comp][q];
          const float2 a = cd[3 * q + 0];
          const float2 b = cd[3 * q + 1];
          const float2 z = cd[3 * q + 2];
          phi = phi + a.x * Tq.x;
          TA[q].x = (b.x * Tq.x - b.y * Tq.y) + z.x * Eold;
          TA[q].y = (b.x * Tq.y + b.y * Tq.x) + z.y * Eold;
        }
        F = c.x * Eold + t1 - t2 - Cs[mm] * phi;
      }
    }
    if (PK != PML_NONE && pml) {
      const float c4 = Cs[mm];
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
    if (src) F = apply_e_sources(F, comp, i, j, k, it, Cs[mm], p);
    e[comp] = F;
    if (NP > 0 && mainu) {
      const float2* cd = CD + mm * 3 * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float2 z = cd[3 * q + 2];
        t[comp][q].x = TA[q].x - z.x * F;
        t[comp][q].y = TA[q].y - z.y * F;
      }
    }
  }
}

// E half-step. Domain: i in [0, nx), j in [0, ny), k in [0, nz). NP = dispersive poles.
template <int PK, int NP, int IDP>
__global__ void __launch_bounds__(kThreads, NP >= 3 ? 3 : 4)
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
  const int nx = p.nx, ny = p.ny, nz = p.nz, sx = p.sx, sy = p.sy;
  const float* __restrict__ Hx = p.H[0];
  const float* __restrict__ Hy = p.H[1];
  const float* __restrict__ Hz = p.H[2];
  constexpr int NPV = NP > 0 ? NP : 1;
  const long long total = (long long)nx * sx;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  FlatWalk w(q, stride, sx, sy, ny + 1);
  // interior box: nodes outside every E slab range (minus [1,T], plus [n-T, n-1])
  const int xlo = p.slab[0].T, xhi = nx - p.slab[3].T;
  const int ylo = p.slab[1].T, yhi = ny - p.slab[4].T;
  const int zlo = p.slab[2].T, zhi = nz - p.slab[5].T;
  int it = 0;
  if (p.nsrcE) it = *p.d_it;
  for (; q < total; q += stride, w.advance(sy)) {
    const int idx = (int)q;
    const int i = w.i, j = w.j, k = w.k;
    if (j >= ny || k >= nz) continue;
    // issue every load of the node before any store
    const float hx_c = __ldg(Hx + idx), hy_c = __ldg(Hy + idx), hz_c = __ldg(Hz + idx);
    const float hx_j = j >= 1 ? __ldg(Hx + idx - sy) : 0.f;
    const float hz_j = j >= 1 ? __ldg(Hz + idx - sy) : 0.f;
    const float hx_k = k >= 1 ? __ldg(Hx + idx - 1) : 0.f;
    const float hy_k = k >= 1 ? __ldg(Hy + idx - 1) : 0.f;
    const float hy_p = i >= 1 ? __ldg(Hy + idx - sx) : 0.f;
    const float hz_p = i >= 1 ? __ldg(Hz + idx - sx) : 0.f;
    uint32_t m[3];
    float e[3];
    float2 t[3][NPV];
    // dispersive state is identically zero on nodes whose materials have no poles (their
    // coefficients are all zero), so it is not written there; it is still read with the
    // node's other loads, which keeps those loads independent of the ID load
    bool disp = NP > 0;
    if (IDP == 1) {
      const uint32_t w = __ldg(p.PE + idx);
      m[0] = w & kPackMask;
      m[1] = (w >> kPackBits) & kPackMask;
      m[2] = (w >> (2 * kPackBits)) & kPackMask;
      disp = NP > 0 && (w & kDispersiveBit);
    } else {
#pragma unroll
      for (int comp = 0; comp < 3; ++comp) m[comp] = __ldg(p.ID[comp] + idx);
    }
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      e[comp] = p.E[comp][idx];
#pragma unroll
      for (int qq = 0; qq < NP; ++qq) t[comp][qq] = p.T[(comp * NP + qq) * (long long)p.ncomp + idx];
    }
    int px0 = -1, pxmax = -1, py0 = -1, pymax = -1, pz0 = -1, pzmax = -1;
    if (PK != PML_NONE && !(i > xlo && i < xhi && j > ylo && j < yhi && k > zlo && k < zhi)) {
      px0 = slab_p<true>(i, p.slab[0].T, nx, true);
      pxmax = slab_p<true>(i, p.slab[3].T, nx, false);
      py0 = slab_p<true>(j, p.slab[1].T, ny, true);
      pymax = slab_p<true>(j, p.slab[4].T, ny, false);
      pz0 = slab_p<true>(k, p.slab[2].T, nz, true);
      pzmax = slab_p<true>(k, p.slab[5].T, nz, false);
    }
    const bool src = p.nsrcE && node_has_source(idx, p.nsrcE, p.srcqE, p.srcE, sx, sy);
    e_node<PK, NP>(p, C4, Cs, CD, i, j, k, src, it, px0, pxmax, py0, pymax, pz0, pzmax, hz_c - hz_j,
                   hy_c - hy_k, hx_c - hx_k, hz_c - hz_p, hy_c - hy_p, hx_c - hx_j, m, e, t);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      p.E[comp][idx] = e[comp];
      if (disp) {
#pragma unroll
        for (int qq = 0; qq < NP; ++qq) p.T[(comp * NP + qq) * (long long)p.ncomp + idx] = t[comp][qq];
      }
    }
  }
}

#ifndef GBF_KERNELS_ONLY
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

// Packed per-node material words for the half-step kernels (IDs < 1024): E word holds the Ex,
// Ey, Ez IDs and a flag that one of them has dispersive poles; H word the Hx, Hy, Hz IDs.
__global__ void pack_ids(const __grid_constant__ StepParams p, const unsigned char* dispersive,
                         uint32_t* pe, uint32_t* ph) {
  const int n = p.ncomp;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const uint32_t ex = p.ID[0][q], ey = p.ID[1][q], ez = p.ID[2][q];
    uint32_t w = ex | (ey << kPackBits) | (ez << (2 * kPackBits));
    if (dispersive && (dispersive[ex] | dispersive[ey] | dispersive[ez])) w |= kDispersiveBit;
    pe[q] = w;
    ph[q] = p.ID[3][q] | (p.ID[4][q] << kPackBits) | (p.ID[5][q] << (2 * kPackBits));
  }
}
#endif  // GBF_KERNELS_ONLY
}  // namespace gbf
