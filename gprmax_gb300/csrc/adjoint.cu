// adjoint.cu — differentiable time loop: forward kernels with per-edge E coefficients and the
// discrete adjoint (transposed updates, reverse time) with checkpoint-and-recompute.
//
// Model (gprmax_gb300/adjoint.py states it in full): the reference's Yee update
// (fields_updates_ext.pyx update_electric/update_magnetic), HORIPML order-1 slab corrections
// (pml_updates_{electric,magnetic}_HORIPML_ext.pyx order1_*), Hertzian dipoles
// (sources.py:163-193) and field receivers (fields_outputs.py:40-67), with one (CA, CB) pair per
// E edge instead of a material-ID lookup, free-space H coefficients and cubic cells. Phi state is
// stored per slab and tangential component ("pair": x (Ey, Ez), y (Ex, Ez), z (Ex, Ey) for E and
// x (Hy, Hz), y (Hx, Hz), z (Hx, Hy) for H) in the main solver's compact layout.
//
// Backward pass, per segment of K steps (from the last): the forward is recomputed from the
// segment's checkpoint straight into per-step slots (E_n, PhiE_n, H^{n+1/2}), then undone in
// reverse with two kernels per step:
//   adj_e_step(n)  per E node: finish the adjoint of E_{n+1} (transposed H curl of u_H and the
//                  transposed H-PML differences of step n+1, receiver samples n+1), then undo
//                  the E half-step n: u_E = CB/d lamE, lamE <- CA lamE, PML Phi/dF adjoints,
//                  gradient partials dL/dCA += lamE E_n, dL/dCB += lamE (curl/d, PML X, source)
//   adj_h_step(n)  per H node: lamH += transposed E curl of u_E and transposed E-PML
//                  differences, then undo the H half-step n: u_H = DB/d lamH, PML adjoints
// The gradient partials are fp32 over at most ceil(sqrt(T)) steps and then folded into fp64
// (every that many steps and at the end of each segment).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbfdtd.h"
#define GBF_KERNELS_ONLY
#include "fdtd_kernels.cuh"

using namespace gbf;

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjSrcMax = 16;
constexpr int kAdjRxMax = 64;

struct AdjSlab {
  int T;            // thickness (0: absent)
  int ocount;       // Phi values per pair
  const float* R;   // [8][T]: ERA ERB ERE ERF HRA HRB HRE HRF (CFS term 0)
};

// Phi-shaped arrays of one field type: [slab][pair] (nullptr for absent slabs)
struct PhiSet {
  float* p[6][2];
};

struct AdjParams {
  int nx, ny, nz, sx, sy, ncomp;
  float rd;      // 1 / d
  float dbd;     // H curl coefficient DB / d
  float srcm;    // H PML coefficient DB
  AdjSlab slab[6];
  const float* CA;   // [3][ncomp]
  const float* CB;
  int nsrc;
  int src_comp[kAdjSrcMax], src_idx[kAdjSrcMax];
  float src_scale[kAdjSrcMax];
  const float* waves;    // [nsrc][iterations]
  int iterations;
  int nrx;
  int rx_comp[kAdjRxMax], rx_idx[kAdjRxMax];
};

// Node walk of a persistent grid over all (nx+1)(ny+1)(nz+1) nodes (as the main kernels).
struct Walk {
  int i, j, k, si, sj, sk;
  __device__ __forceinline__ Walk(int q, int stride, const AdjParams& p) {
    i = q / p.sx;
    int r = q - i * p.sx;
    j = r / p.sy;
    k = r - j * p.sy;
    si = stride / p.sx;
    r = stride - si * p.sx;
    sj = r / p.sy;
    sk = r - sj * p.sy;
  }
  __device__ __forceinline__ void advance(const AdjParams& p) {
    k += sk;
    if (k >= p.sy) { k -= p.sy; ++j; }
    j += sj;
    if (j > p.ny) { j -= p.ny + 1; ++i; }
    i += si;
  }
};

// pair index (0: first, 1: second tangential component) of component C on slab axis AX, -1 if
// C is not tangential; the sign of the correction (E: x Ey -, Ez +; y Ex +, Ez -; z Ex -, Ey +;
// H the opposite); the component whose difference drives it.
__host__ __device__ constexpr int pair_of(int AX, int C) {
  return AX == 0 ? (C == 1 ? 0 : C == 2 ? 1 : -1)
       : AX == 1 ? (C == 0 ? 0 : C == 2 ? 1 : -1)
                 : (C == 0 ? 0 : C == 1 ? 1 : -1);
}
__host__ __device__ constexpr float pair_sign(bool electric, int AX, int C) {
  return (electric != ((AX == 0) ? (C == 1) : (AX == 1) ? (C == 2) : (C == 0))) ? 1.f : -1.f;
}
__host__ __device__ constexpr int pair_driver(int AX, int C) {
  return AX == 0 ? (C == 1 ? 2 : 1) : AX == 1 ? (C == 0 ? 2 : 0) : (C == 0 ? 1 : 0);
}

__device__ __forceinline__ int axis_stride(int AX, const AdjParams& p) {
  return AX == 0 ? p.sx : AX == 1 ? p.sy : 1;
}

// Slab of axis AX holding node (i, j, k) (E ranges if ELECTRIC, else H ranges; every coordinate
// below its cell count): slab index (-1 if none), profile index and Phi index.
template <bool ELECTRIC, int AX>
__device__ __forceinline__ int slab_of(const AdjParams& p, int i, int j, int k, int& pr,
                                       int& pidx) {
  if (i < 0 || j < 0 || k < 0 || i >= p.nx || j >= p.ny || k >= p.nz) return -1;
  const int c = AX == 0 ? i : AX == 1 ? j : k;
  const int n = AX == 0 ? p.nx : AX == 1 ? p.ny : p.nz;
  const int where = axis_member<ELECTRIC>(c, n, p.slab[AX].T, p.slab[AX + 3].T, pr);
  if (!where) return -1;
  const int s = AX + (where == 2 ? 3 : 0);
  pidx = phi_index<AX>(i, j, k, pr, p.slab[s].T, p.ny, p.nz);
  return s;
}

// Is the node within one cell of any slab (so that it or a neighbour may be in one)?
__device__ __forceinline__ bool near_slab(const AdjParams& p, int i, int j, int k) {
  return i <= p.slab[0].T + 1 || i >= p.nx - p.slab[3].T - 1 ||
         j <= p.slab[1].T + 1 || j >= p.ny - p.slab[4].T - 1 ||
         k <= p.slab[2].T + 1 || k >= p.nz - p.slab[5].T - 1;
}

__device__ __forceinline__ bool e_updated(int C, int i, int j, int k, const AdjParams& p) {
  if (C == 0) return i < p.nx && j >= 1 && j < p.ny && k >= 1 && k < p.nz;
  if (C == 1) return i >= 1 && i < p.nx && j < p.ny && k >= 1 && k < p.nz;
  return i >= 1 && i < p.nx && j >= 1 && j < p.ny && k < p.nz;
}

__device__ __forceinline__ bool h_updated(int C, int i, int j, int k, const AdjParams& p) {
  if (C == 0) return i >= 1 && j < p.ny && k < p.nz;
  if (C == 1) return i < p.nx && j >= 1 && k < p.nz;
  return i < p.nx && j < p.ny && k >= 1;
}

// E curl bracket of component C at idx (multiplied by CB/d in the update)
__device__ __forceinline__ float e_curl(int C, int idx, const float* H, const AdjParams& p) {
  const float* Hx = H;
  const float* Hy = H + p.ncomp;
  const float* Hz = H + 2 * (size_t)p.ncomp;
  if (C == 0) return (Hz[idx] - Hz[idx - p.sy]) - (Hy[idx] - Hy[idx - 1]);
  if (C == 1) return (Hx[idx] - Hx[idx - 1]) - (Hz[idx] - Hz[idx - p.sx]);
  return (Hy[idx] - Hy[idx - p.sx]) - (Hx[idx] - Hx[idx - p.sy]);
}

// slab corrections of component C in the reference's slab order (x0 y0 z0 xmax ymax zmax):
// axis b before a (a < b) only when a's slab is a plus slab and b's a minus slab
template <int C>
__device__ __forceinline__ float apply_terms(float F, const int* s, const float* t) {
  constexpr int a = C == 0 ? 1 : 0;
  constexpr int b = C == 2 ? 1 : 2;
  if (s[a] >= 3 && s[b] >= 0 && s[b] < 3) {
    F = F + t[b];
    F = F + t[a];
  } else {
    if (s[a] >= 0) F = F + t[a];
    if (s[b] >= 0) F = F + t[b];
  }
  return F;
}

// ---- forward --------------------------------------------------------------------------
// H half-step: Hout = update(Hin, E); Phi_H in place. Hin may equal Hout.
__global__ void __launch_bounds__(kAdjThreads)
adj_fwd_h(const __grid_constant__ AdjParams p, const float* __restrict__ E, const float* Hin,
          float* Hout, const __grid_constant__ PhiSet phi) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.ncomp) return;
  Walk w(q, stride, p);
  const float* Ex = E;
  const float* Ey = E + p.ncomp;
  const float* Ez = E + 2 * (size_t)p.ncomp;
  for (; q < p.ncomp; q += stride, w.advance(p)) {
    const int i = w.i, j = w.j, k = w.k, idx = q;
    float h[3];
#pragma unroll
    for (int C = 0; C < 3; ++C) h[C] = Hin[C * (size_t)p.ncomp + idx];
    if (h_updated(0, i, j, k, p))
      h[0] = h[0] - p.dbd * (Ez[idx + p.sy] - Ez[idx]) + p.dbd * (Ey[idx + 1] - Ey[idx]);
    if (h_updated(1, i, j, k, p))
      h[1] = h[1] - p.dbd * (Ex[idx + 1] - Ex[idx]) + p.dbd * (Ez[idx + p.sx] - Ez[idx]);
    if (h_updated(2, i, j, k, p))
      h[2] = h[2] - p.dbd * (Ey[idx + p.sx] - Ey[idx]) + p.dbd * (Ex[idx + p.sy] - Ex[idx]);
    if (near_slab(p, i, j, k)) {
      int s[3], pr[3], pidx[3];
      s[0] = slab_of<false, 0>(p, i, j, k, pr[0], pidx[0]);
      s[1] = slab_of<false, 1>(p, i, j, k, pr[1], pidx[1]);
      s[2] = slab_of<false, 2>(p, i, j, k, pr[2], pidx[2]);
      float t[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // [component][axis]
#pragma unroll
      for (int AX = 0; AX < 3; ++AX) {
        if (s[AX] < 0) continue;
        const AdjSlab& sl = p.slab[s[AX]];
        const int T = sl.T, r = pr[AX];
        const float RA = sl.R[4 * T + r], RB = sl.R[5 * T + r], RE = sl.R[6 * T + r], RF = sl.R[7 * T + r];
        const int st = axis_stride(AX, p);
#pragma unroll
        for (int C = 0; C < 3; ++C) {
          const int pw = pair_of(AX, C);
          if (pw < 0) continue;
          const float* D = E + pair_driver(AX, C) * (size_t)p.ncomp;
          const float dF = (D[idx + st] - D[idx]) * p.rd;
          float* ph = phi.p[s[AX]][pw] + pidx[AX];
          const float v = *ph;
          const float X = (RA - 1.0f) * dF + RB * v;
          *ph = RE * v - RF * dF;
          t[C][AX] = pair_sign(false, AX, C) * (p.srcm * X);
        }
      }
      h[0] = apply_terms<0>(h[0], s, t[0]);
      h[1] = apply_terms<1>(h[1], s, t[1]);
      h[2] = apply_terms<2>(h[2], s, t[2]);
    }
#pragma unroll
    for (int C = 0; C < 3; ++C) Hout[C * (size_t)p.ncomp + idx] = h[C];
  }
}

// E half-step n: Eout = update(Ein, H); Phi_E read from phin, written to phout; sources.
// Ein may equal Eout and phin phout.
__global__ void __launch_bounds__(kAdjThreads)
adj_fwd_e(const __grid_constant__ AdjParams p, const float* Ein, float* Eout,
          const float* __restrict__ H, const __grid_constant__ PhiSet phin,
          const __grid_constant__ PhiSet phout, int it) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.ncomp) return;
  Walk w(q, stride, p);
  for (; q < p.ncomp; q += stride, w.advance(p)) {
    const int i = w.i, j = w.j, k = w.k, idx = q;
    float e[3], cb[3];
#pragma unroll
    for (int C = 0; C < 3; ++C) {
      const size_t o = C * (size_t)p.ncomp + idx;
      e[C] = Ein[o];
      cb[C] = p.CB[o];
      if (e_updated(C, i, j, k, p)) e[C] = p.CA[o] * e[C] + (cb[C] * p.rd) * e_curl(C, idx, H, p);
    }
    if (near_slab(p, i, j, k)) {
      int s[3], pr[3], pidx[3];
      s[0] = slab_of<true, 0>(p, i, j, k, pr[0], pidx[0]);
      s[1] = slab_of<true, 1>(p, i, j, k, pr[1], pidx[1]);
      s[2] = slab_of<true, 2>(p, i, j, k, pr[2], pidx[2]);
      float t[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
      for (int AX = 0; AX < 3; ++AX) {
        if (s[AX] < 0) continue;
        const AdjSlab& sl = p.slab[s[AX]];
        const int T = sl.T, r = pr[AX];
        const float RA = sl.R[r], RB = sl.R[T + r], RE = sl.R[2 * T + r], RF = sl.R[3 * T + r];
        const int st = axis_stride(AX, p);
#pragma unroll
        for (int C = 0; C < 3; ++C) {
          const int pw = pair_of(AX, C);
          if (pw < 0) continue;
          const float* D = H + pair_driver(AX, C) * (size_t)p.ncomp;
          const float dF = (D[idx] - D[idx - st]) * p.rd;
          const float v = phin.p[s[AX]][pw][pidx[AX]];
          const float X = (RA - 1.0f) * dF + RB * v;
          phout.p[s[AX]][pw][pidx[AX]] = RE * v - RF * dF;
          t[C][AX] = pair_sign(true, AX, C) * (cb[C] * X);
        }
      }
      e[0] = apply_terms<0>(e[0], s, t[0]);
      e[1] = apply_terms<1>(e[1], s, t[1]);
      e[2] = apply_terms<2>(e[2], s, t[2]);
    }
    for (int n = 0; n < p.nsrc; ++n)
      if (p.src_idx[n] == idx) {
        const int C = p.src_comp[n];
        e[C] = e[C] - cb[C] * p.waves[(size_t)n * p.iterations + it] * p.src_scale[n];
      }
#pragma unroll
    for (int C = 0; C < 3; ++C) Eout[C * (size_t)p.ncomp + idx] = e[C];
  }
}

__global__ void adj_fwd_rx(const __grid_constant__ AdjParams p, const float* E, float* traces, int it) {
  for (int r = threadIdx.x; r < p.nrx; r += blockDim.x)
    traces[(size_t)r * p.iterations + it] = E[p.rx_comp[r] * (size_t)p.ncomp + p.rx_idx[r]];
}

// ---- adjoint --------------------------------------------------------------------------
struct AdjStep {
  float* lE;          // [3][ncomp] adjoint of E (in place)
  float* lH;          // [3][ncomp] adjoint of H (in place)
  float* uE;          // [3][ncomp]
  float* uH;          // [3][ncomp]
  PhiSet lphiE, lphiH, dFE, dFH;
  const float* En;    // forward E_n
  const float* Hh;    // forward H^{n+1/2}
  PhiSet PEn;         // forward Phi_E at step n
  float* gCA;         // [3][ncomp] fp32 partials of the segment
  float* gCB;
  const float* gtr;   // [nrx][iterations] d(misfit)/d(traces)
  int it;             // step being undone (n)
  int finish;         // 1: lamE still needs the step n+1 terms (n + 1 < iterations)
};

__device__ __forceinline__ float at(const float* a, int C, int i, int j, int k, const AdjParams& p) {
  if (i < 0 || j < 0 || k < 0 || i > p.nx || j > p.ny || k > p.nz) return 0.f;
  return a[C * (size_t)p.ncomp + i * p.sx + j * p.sy + k];
}

template <bool ELECTRIC, int AX>
__device__ __forceinline__ float dF_at(const PhiSet& d, int C, int i, int j, int k,
                                       const AdjParams& p) {
  int pr, pidx;
  const int s = slab_of<ELECTRIC, AX>(p, i, j, k, pr, pidx);
  return s < 0 ? 0.f : d.p[s][pair_of(AX, C)][pidx];
}

// Both adjoint kernels wait on memory latency (each node's some forty loads: forward state,
// coefficients, adjoint state, partials), so they run 5 blocks of 256 per SM at 48 registers
// rather than 4 at 64: gradient of the 200 x 200 x 100 workload 0.970 s against 1.074 s (6
// blocks, with spills: 1.008 s).
__global__ void __launch_bounds__(kAdjThreads, 5)
adj_e_step(const __grid_constant__ AdjParams p, const __grid_constant__ AdjStep b) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.ncomp) return;
  Walk w(q, stride, p);
  const float rd = p.rd;
  for (; q < p.ncomp; q += stride, w.advance(p)) {
    const int i = w.i, j = w.j, k = w.k, idx = q;
    float lam[3];
#pragma unroll
    for (int C = 0; C < 3; ++C) lam[C] = b.lE[C * (size_t)p.ncomp + idx];
    const bool near = near_slab(p, i, j, k);
    if (b.finish) {
      // adjoint of E_{n+1}: transposed H curl of u_H (Hx -= DB/d (Ez(j+1) - Ez) - DB/d (Ey(k+1) - Ey) ...)
      const float* u = b.uH;
      lam[0] += at(u, 1, i, j, k, p) - at(u, 1, i, j, k - 1, p) + at(u, 2, i, j - 1, k, p) - at(u, 2, i, j, k, p);
      lam[1] += at(u, 0, i, j, k - 1, p) - at(u, 0, i, j, k, p) - at(u, 2, i - 1, j, k, p) + at(u, 2, i, j, k, p);
      lam[2] += -at(u, 0, i, j - 1, k, p) + at(u, 0, i, j, k, p) + at(u, 1, i - 1, j, k, p) - at(u, 1, i, j, k, p);
      if (near) {
        // H-PML differences dF(h) = (E(h + a) - E(h)) / d feed E at h + a and h
        lam[2] += rd * (dF_at<false, 0>(b.dFH, 1, i - 1, j, k, p) - dF_at<false, 0>(b.dFH, 1, i, j, k, p) +
                        dF_at<false, 1>(b.dFH, 0, i, j - 1, k, p) - dF_at<false, 1>(b.dFH, 0, i, j, k, p));
        lam[1] += rd * (dF_at<false, 0>(b.dFH, 2, i - 1, j, k, p) - dF_at<false, 0>(b.dFH, 2, i, j, k, p) +
                        dF_at<false, 2>(b.dFH, 0, i, j, k - 1, p) - dF_at<false, 2>(b.dFH, 0, i, j, k, p));
        lam[0] += rd * (dF_at<false, 1>(b.dFH, 2, i, j - 1, k, p) - dF_at<false, 1>(b.dFH, 2, i, j, k, p) +
                        dF_at<false, 2>(b.dFH, 1, i, j, k - 1, p) - dF_at<false, 2>(b.dFH, 1, i, j, k, p));
      }
      for (int r = 0; r < p.nrx; ++r)
        if (p.rx_idx[r] == idx) lam[p.rx_comp[r]] += b.gtr[(size_t)r * p.iterations + b.it + 1];
    }
    // undo the E half-step n
    float gcb[3] = {0.f, 0.f, 0.f};
    float cb[3];
#pragma unroll
    for (int C = 0; C < 3; ++C) {
      const size_t o = C * (size_t)p.ncomp + idx;
      cb[C] = p.CB[o];
      float u = 0.f, lnew = lam[C];
      if (e_updated(C, i, j, k, p)) {
        u = (cb[C] * rd) * lam[C];
        lnew = p.CA[o] * lam[C];
        b.gCA[o] += lam[C] * b.En[o];
        gcb[C] = lam[C] * (rd * e_curl(C, idx, b.Hh, p));
      }
      b.uE[o] = u;
      b.lE[o] = lnew;
    }
    if (near) {
      int s[3], pr[3], pidx[3];
      s[0] = slab_of<true, 0>(p, i, j, k, pr[0], pidx[0]);
      s[1] = slab_of<true, 1>(p, i, j, k, pr[1], pidx[1]);
      s[2] = slab_of<true, 2>(p, i, j, k, pr[2], pidx[2]);
#pragma unroll
      for (int AX = 0; AX < 3; ++AX) {
        if (s[AX] < 0) continue;
        const AdjSlab& sl = p.slab[s[AX]];
        const int T = sl.T, r = pr[AX];
        const float RA = sl.R[r], RB = sl.R[T + r], RE = sl.R[2 * T + r], RF = sl.R[3 * T + r];
        const int st = axis_stride(AX, p);
#pragma unroll
        for (int C = 0; C < 3; ++C) {
          const int pw = pair_of(AX, C);
          if (pw < 0) continue;
          const int o = pidx[AX];
          const float sg = pair_sign(true, AX, C);
          const float Xb = sg * cb[C] * lam[C];
          float* lph = b.lphiE.p[s[AX]][pw] + o;
          const float l0 = *lph;
          b.dFE.p[s[AX]][pw][o] = (RA - 1.0f) * Xb - RF * l0;
          *lph = RB * Xb + RE * l0;
          const float* D = b.Hh + pair_driver(AX, C) * (size_t)p.ncomp;
          const float dF = (D[idx] - D[idx - st]) * rd;
          const float X = (RA - 1.0f) * dF + RB * b.PEn.p[s[AX]][pw][o];
          gcb[C] += sg * X * lam[C];
        }
      }
    }
    for (int n = 0; n < p.nsrc; ++n)
      if (p.src_idx[n] == idx) {
        const int C = p.src_comp[n];
        gcb[C] -= p.waves[(size_t)n * p.iterations + b.it] * p.src_scale[n] * lam[C];
      }
#pragma unroll
    for (int C = 0; C < 3; ++C) b.gCB[C * (size_t)p.ncomp + idx] += gcb[C];
  }
}

__global__ void __launch_bounds__(kAdjThreads, 5)
adj_h_step(const __grid_constant__ AdjParams p, const __grid_constant__ AdjStep b) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.ncomp) return;
  Walk w(q, stride, p);
  const float rd = p.rd;
  const float* u = b.uE;
  for (; q < p.ncomp; q += stride, w.advance(p)) {
    const int i = w.i, j = w.j, k = w.k, idx = q;
    float lam[3];
#pragma unroll
    for (int C = 0; C < 3; ++C) lam[C] = b.lH[C * (size_t)p.ncomp + idx];
    // transposed E curl (Ex += CB/d ((Hz - Hz(j-1)) - (Hy - Hy(k-1))) ...)
    lam[0] += at(u, 1, i, j, k, p) - at(u, 1, i, j, k + 1, p) - at(u, 2, i, j, k, p) + at(u, 2, i, j + 1, k, p);
    lam[1] += -at(u, 0, i, j, k, p) + at(u, 0, i, j, k + 1, p) + at(u, 2, i, j, k, p) - at(u, 2, i + 1, j, k, p);
    lam[2] += at(u, 0, i, j, k, p) - at(u, 0, i, j + 1, k, p) - at(u, 1, i, j, k, p) + at(u, 1, i + 1, j, k, p);
    const bool near = near_slab(p, i, j, k);
    if (near) {
      // E-PML differences dF(e) = (H(e) - H(e - a)) / d feed H at e and e - a
      lam[2] += rd * (dF_at<true, 0>(b.dFE, 1, i, j, k, p) - dF_at<true, 0>(b.dFE, 1, i + 1, j, k, p) +
                      dF_at<true, 1>(b.dFE, 0, i, j, k, p) - dF_at<true, 1>(b.dFE, 0, i, j + 1, k, p));
      lam[1] += rd * (dF_at<true, 0>(b.dFE, 2, i, j, k, p) - dF_at<true, 0>(b.dFE, 2, i + 1, j, k, p) +
                      dF_at<true, 2>(b.dFE, 0, i, j, k, p) - dF_at<true, 2>(b.dFE, 0, i, j, k + 1, p));
      lam[0] += rd * (dF_at<true, 1>(b.dFE, 2, i, j, k, p) - dF_at<true, 1>(b.dFE, 2, i, j + 1, k, p) +
                      dF_at<true, 2>(b.dFE, 1, i, j, k, p) - dF_at<true, 2>(b.dFE, 1, i, j, k + 1, p));
    }
    // undo the H half-step n (DA = 1: lamH passes through)
#pragma unroll
    for (int C = 0; C < 3; ++C) {
      const size_t o = C * (size_t)p.ncomp + idx;
      b.lH[o] = lam[C];
      b.uH[o] = h_updated(C, i, j, k, p) ? p.dbd * lam[C] : 0.f;
    }
    if (near) {
      int s[3], pr[3], pidx[3];
      s[0] = slab_of<false, 0>(p, i, j, k, pr[0], pidx[0]);
      s[1] = slab_of<false, 1>(p, i, j, k, pr[1], pidx[1]);
      s[2] = slab_of<false, 2>(p, i, j, k, pr[2], pidx[2]);
#pragma unroll
      for (int AX = 0; AX < 3; ++AX) {
        if (s[AX] < 0) continue;
        const AdjSlab& sl = p.slab[s[AX]];
        const int T = sl.T, r = pr[AX];
        const float RA = sl.R[4 * T + r], RB = sl.R[5 * T + r], RE = sl.R[6 * T + r], RF = sl.R[7 * T + r];
#pragma unroll
        for (int C = 0; C < 3; ++C) {
          const int pw = pair_of(AX, C);
          if (pw < 0) continue;
          const int o = pidx[AX];
          const float Xb = pair_sign(false, AX, C) * p.srcm * lam[C];
          float* lph = b.lphiH.p[s[AX]][pw] + o;
          const float l0 = *lph;
          b.dFH.p[s[AX]][pw][o] = (RA - 1.0f) * Xb - RF * l0;
          *lph = RB * Xb + RE * l0;
        }
      }
    }
  }
}

// Add the fp32 partial sums to the fp64 gradient and clear them for the next span.
__global__ void adj_fold(float* __restrict__ a, double* __restrict__ g, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    g[q] += (double)a[q];
    a[q] = 0.f;
  }
}

}  // namespace

// ---- host side -------------------------------------------------------------------------
struct gbf_adj {
  gbf_adj_desc d;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long N = 0;           // nodes per component
  int K = 1;                 // recompute slots (the longest segment)
  int nck = 0;               // checkpoints (segments)
  std::vector<int> seg;      // segment starts, nck + 1 entries (the last is iterations)
  size_t phi_len = 0;        // floats of one PhiSet (every slab, both pairs)
  size_t off[6] = {0, 0, 0, 0, 0, 0};
  AdjParams p{};
  std::vector<void*> allocs;
  float* pml_rows = nullptr; // 6 x 8 x Tmax
  float* waves = nullptr;
  float *E = nullptr, *H = nullptr, *phiE = nullptr, *phiH = nullptr;   // forward state
  float* ckpt = nullptr;     // nck x (6N + 2 phi_len)
  float *segE = nullptr, *segPhiE = nullptr, *segH = nullptr;         // recompute slots
  float *recH = nullptr, *recPhiH = nullptr;
  float *lE = nullptr, *lH = nullptr, *uE = nullptr, *uH = nullptr;
  float *lphiE = nullptr, *lphiH = nullptr, *dFE = nullptr, *dFH = nullptr;
  float *gCA = nullptr, *gCB = nullptr;                                // fp32 segment partials
  bool forward_done = false;
  bool resident = false;     // the slots hold the last segment's states from the forward
  int grid = 0;      // persistent grid of the forward kernels (and the folds)
  int grid_be = 0, grid_bh = 0;   // of the two adjoint kernels
};

static std::string g_adj_err;

static int afail(gbf_adj* a, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (a) a->err = buf;
  else g_adj_err = buf;
  return code;
}

#define AK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return afail(a, e_ == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA,           \
                   "%s failed: %s", #call, cudaGetErrorString(e_));                       \
  } while (0)

static PhiSet phiset(const gbf_adj* a, float* base) {
  PhiSet ps;
  for (int s = 0; s < 6; ++s) {
    const int oc = a->p.slab[s].ocount;
    ps.p[s][0] = (a->p.slab[s].T && base) ? base + a->off[s] : nullptr;
    ps.p[s][1] = (a->p.slab[s].T && base) ? base + a->off[s] + oc : nullptr;
  }
  return ps;
}

static int copy_d2d(gbf_adj* a, float* dst, const float* src, size_t n) {
  if (n) AK(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, a->stream));
  return GBF_OK;
}

extern "C" {

int gbf_adj_create(const gbf_adj_desc* desc, gbf_adj** out) {
  if (!desc || !out) return afail(nullptr, GBF_EINVAL, "gbf_adj_create: null argument");
  *out = nullptr;
  const gbf_adj_desc& d = *desc;
  if (d.nx < 2 || d.ny < 2 || d.nz < 2 || d.iterations < 1)
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: 3D grid and at least one iteration needed");
  if (!(d.d > 0.f) || !(d.dt > 0.f))
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: cell size and time step must be positive");
  if (d.nsrc < 0 || d.nsrc > kAdjSrcMax || d.nrx < 1 || d.nrx > kAdjRxMax)
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: 0..%d sources and 1..%d receivers", kAdjSrcMax, kAdjRxMax);
  if (d.checkpoint_interval < -1 || d.reserved[0] || d.reserved[1] || d.reserved[2])
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: bad checkpoint interval or reserved fields");
  const int n3[3] = {d.nx, d.ny, d.nz};
  for (int s = 0; s < 6; ++s)
    if (d.pml_thickness[s] < 0 || 2 * d.pml_thickness[s] >= n3[s % 3])
      return afail(nullptr, GBF_EINVAL, "gbf_adj_create: PML slab %d thickness %d too large", s, d.pml_thickness[s]);
  const long long N = (long long)(d.nx + 1) * (d.ny + 1) * (d.nz + 1);
  if (N > (1LL << 31) - 1) return afail(nullptr, GBF_EINVAL, "gbf_adj_create: more than 2^31 nodes");
  gbf_adj* a = new gbf_adj();
  a->d = d;
  a->N = N;
  a->K = d.checkpoint_interval > 0 ? d.checkpoint_interval : (int)ceil(sqrt((double)d.iterations));
  if (a->K > d.iterations) a->K = d.iterations;
  a->nck = (d.iterations + a->K - 1) / a->K;
  cudaError_t e = cudaGetDevice(&a->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    afail(nullptr, GBF_ECUDA, "gbf_adj_create: CUDA unavailable: %s", cudaGetErrorString(e));
    delete a;
    return GBF_ECUDA;
  }
  AdjParams& p = a->p;
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  p.sy = d.nz + 1;
  p.sx = (d.ny + 1) * (d.nz + 1);
  p.ncomp = (int)N;
  p.rd = 1.0f / d.d;
  p.dbd = d.dbd;
  p.srcm = d.srcm;
  p.iterations = d.iterations;
  int Tmax = 1;
  for (int s = 0; s < 6; ++s) {
    const int t = d.pml_thickness[s];
    Tmax = t > Tmax ? t : Tmax;
    const int ax = s % 3;
    const long long nu = ax == 0 ? d.ny : d.nx, nv = ax == 2 ? d.ny : d.nz;
    p.slab[s].T = t;
    p.slab[s].ocount = t ? (int)(t * nu * nv) : 0;
    a->off[s] = a->phi_len;
    a->phi_len += 2 * (size_t)p.slab[s].ocount;
  }
  // segments: every K steps; with interval -1 the last segment is as long as the recompute
  // slots (E, H and the E-side PML state per step) that fit in 60 % of the free device memory
  // (the forward leaves it in the slots, so only the steps before it are ever recomputed), and
  // the steps before it form segments of ceil(sqrt(their count))
  {
    const int T = d.iterations;
    int last = T - (a->nck - 1) * a->K;
    if (d.checkpoint_interval == -1) {
      size_t freeb = 0, totalb = 0;
      if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) freeb = 0;
      const double per_step = 4.0 * (6.0 * (double)N + (double)a->phi_len);
      long long l = (long long)(0.6 * (double)freeb / per_step);
      if (l > T) l = T;
      if (l < a->K) l = a->K < T ? a->K : T;
      last = (int)l;
      const int rest = T - last;
      const int k0 = rest > 0 ? (int)ceil(sqrt((double)rest)) : 1;
      a->seg.clear();
      for (int s0 = 0; s0 < rest; s0 += k0) a->seg.push_back(s0);
      a->seg.push_back(rest);
      a->seg.push_back(T);
      a->K = last > k0 ? last : k0;
    } else {
      a->seg.clear();
      for (int s0 = 0; s0 < T; s0 += a->K) a->seg.push_back(s0);
      a->seg.push_back(T);
    }
    a->nck = (int)a->seg.size() - 1;
  }
  const size_t PL = a->phi_len, K = a->K;
  const size_t ck = 6 * (size_t)N + 2 * PL;
  int rc = GBF_OK;
  auto A = [&](float** ptr, size_t floats) {
    if (rc != GBF_OK) return;
    cudaError_t r = cudaMalloc((void**)ptr, sizeof(float) * (floats ? floats : 1));
    if (r != cudaSuccess) {
      rc = afail(a, r == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA, "gbf_adj_create: allocation of %zu bytes failed: %s",
                 sizeof(float) * floats, cudaGetErrorString(r));
      return;
    }
    a->allocs.push_back(*ptr);
    r = cudaMemsetAsync(*ptr, 0, sizeof(float) * (floats ? floats : 1), a->stream);
    if (r != cudaSuccess) rc = afail(a, GBF_ECUDA, "gbf_adj_create: %s", cudaGetErrorString(r));
  };
  A(&a->pml_rows, 6 * 8 * (size_t)Tmax);
  A(&a->waves, (size_t)(d.nsrc + 1) * d.iterations);
  A(&a->E, 3 * (size_t)N);
  A(&a->H, 3 * (size_t)N);
  A(&a->phiE, PL);
  A(&a->phiH, PL);
  A(&a->ckpt, ck * a->nck);
  A(&a->segE, 3 * (size_t)N * (K + 1));
  A(&a->segPhiE, PL * (K + 1));
  A(&a->segH, 3 * (size_t)N * K);
  A(&a->recH, 3 * (size_t)N);
  A(&a->recPhiH, PL);
  A(&a->lE, 3 * (size_t)N);
  A(&a->lH, 3 * (size_t)N);
  A(&a->uE, 3 * (size_t)N);
  A(&a->uH, 3 * (size_t)N);
  A(&a->lphiE, PL);
  A(&a->lphiH, PL);
  A(&a->dFE, PL);
  A(&a->dFH, PL);
  A(&a->gCA, 3 * (size_t)N);
  A(&a->gCB, 3 * (size_t)N);
  if (rc != GBF_OK) {
    g_adj_err = a->err;
    gbf_adj_destroy(a);
    return rc;
  }
  for (int s = 0; s < 6; ++s) p.slab[s].R = a->pml_rows + (size_t)s * 8 * Tmax;
  p.waves = a->waves;
  int dev = 0, sms = 1, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // each group of kernels on as many blocks as its occupancy keeps resident
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, adj_fwd_e, kAdjThreads, 0);
  a->grid = sms * (per > 0 ? per : 1);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, adj_e_step, kAdjThreads, 0);
  a->grid_be = sms * (per > 0 ? per : 1);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, adj_h_step, kAdjThreads, 0);
  a->grid_bh = sms * (per > 0 ? per : 1);
  *out = a;
  return GBF_OK;
}

void gbf_adj_destroy(gbf_adj* a) {
  if (!a) return;
  if (a->stream) cudaStreamSynchronize(a->stream);
  for (void* q : a->allocs) cudaFree(q);
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
}

int gbf_adj_last_error(gbf_adj* a, char* buf, size_t n) {
  if (!buf || n == 0) return GBF_EINVAL;
  snprintf(buf, n, "%s", a ? a->err.c_str() : g_adj_err.c_str());
  return GBF_OK;
}

int gbf_adj_upload_pml(gbf_adj* a, int32_t slab, const float* const rows[8]) {
  if (!a || slab < 0 || slab > 5 || !rows) return GBF_EINVAL;
  const int T = a->d.pml_thickness[slab];
  if (!T) return afail(a, GBF_EINVAL, "gbf_adj_upload_pml: slab %d has zero thickness", slab);
  for (int r = 0; r < 8; ++r) {
    if (!rows[r]) return afail(a, GBF_EINVAL, "gbf_adj_upload_pml: row %d missing", r);
    AK(cudaMemcpyAsync(const_cast<float*>(a->p.slab[slab].R) + (size_t)r * T, rows[r],
                       sizeof(float) * T, cudaMemcpyHostToDevice, a->stream));
  }
  AK(cudaStreamSynchronize(a->stream));
  return GBF_OK;
}

int gbf_adj_upload_sources(gbf_adj* a, const int32_t* info, const float* scale, const float* waves) {
  if (!a) return GBF_EINVAL;
  const gbf_adj_desc& d = a->d;
  if (d.nsrc && (!info || !scale || !waves)) return GBF_EINVAL;
  for (int s = 0; s < d.nsrc; ++s) {
    const int C = info[4 * s], i = info[4 * s + 1], j = info[4 * s + 2], k = info[4 * s + 3];
    if (C < 0 || C > 2 || i < 0 || j < 0 || k < 0 || i > d.nx || j > d.ny || k > d.nz)
      return afail(a, GBF_EINVAL, "gbf_adj_upload_sources: source %d out of the grid", s);
    a->p.src_comp[s] = C;
    a->p.src_idx[s] = i * a->p.sx + j * a->p.sy + k;
    a->p.src_scale[s] = scale[s];
  }
  a->p.nsrc = d.nsrc;
  if (d.nsrc)
    AK(cudaMemcpyAsync(a->waves, waves, sizeof(float) * (size_t)d.nsrc * d.iterations,
                       cudaMemcpyHostToDevice, a->stream));
  AK(cudaStreamSynchronize(a->stream));
  return GBF_OK;
}

int gbf_adj_set_receivers(gbf_adj* a, const int32_t* info) {
  if (!a || !info) return GBF_EINVAL;
  const gbf_adj_desc& d = a->d;
  for (int r = 0; r < d.nrx; ++r) {
    const int C = info[4 * r], i = info[4 * r + 1], j = info[4 * r + 2], k = info[4 * r + 3];
    if (C < 0 || C > 2 || i < 0 || j < 0 || k < 0 || i > d.nx || j > d.ny || k > d.nz)
      return afail(a, GBF_EINVAL, "gbf_adj_set_receivers: receiver %d out of the grid", r);
    a->p.rx_comp[r] = C;
    a->p.rx_idx[r] = i * a->p.sx + j * a->p.sy + k;
  }
  a->p.nrx = d.nrx;
  return GBF_OK;
}

int gbf_adj_forward(gbf_adj* a, const float* CA, const float* CB, float* traces) {
  if (!a || !CA || !CB || !traces) return GBF_EINVAL;
  if (!a->p.nrx) return afail(a, GBF_ESTATE, "gbf_adj_forward: receivers not set");
  const size_t N = a->N, PL = a->phi_len, ck = 6 * N + 2 * PL;
  a->p.CA = CA;
  a->p.CB = CB;
  AK(cudaMemsetAsync(a->E, 0, sizeof(float) * 3 * N, a->stream));
  AK(cudaMemsetAsync(a->H, 0, sizeof(float) * 3 * N, a->stream));
  if (PL) AK(cudaMemsetAsync(a->phiE, 0, sizeof(float) * PL, a->stream));
  if (PL) AK(cudaMemsetAsync(a->phiH, 0, sizeof(float) * PL, a->stream));
  const PhiSet pE = phiset(a, a->phiE), pH = phiset(a, a->phiH);
  // the last segment runs straight into the recompute slots (out of place, as the backward
  // would recompute it from its checkpoint), so the backward needs no recompute for it
  const int T = a->d.iterations;
  const int last0 = a->seg[a->nck - 1];
  int sc = 0;   // next segment whose start takes a checkpoint
  for (int it = 0; it < last0; ++it) {
    if (it == a->seg[sc]) {
      float* c = a->ckpt + (size_t)(sc++) * ck;
      int rc = copy_d2d(a, c, a->E, 3 * N);
      if (!rc) rc = copy_d2d(a, c + 3 * N, a->H, 3 * N);
      if (!rc) rc = copy_d2d(a, c + 6 * N, a->phiE, PL);
      if (!rc) rc = copy_d2d(a, c + 6 * N + PL, a->phiH, PL);
      if (rc) return rc;
    }
    adj_fwd_rx<<<1, 64, 0, a->stream>>>(a->p, a->E, traces, it);
    adj_fwd_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, a->E, a->H, a->H, pH);
    adj_fwd_e<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, a->E, a->E, a->H, pE, pE, it);
  }
  {
    float* c = a->ckpt + (size_t)(a->nck - 1) * ck;
    int rc = copy_d2d(a, c, a->E, 3 * N);
    if (!rc) rc = copy_d2d(a, c + 3 * N, a->H, 3 * N);
    if (!rc) rc = copy_d2d(a, c + 6 * N, a->phiE, PL);
    if (!rc) rc = copy_d2d(a, c + 6 * N + PL, a->phiH, PL);
    if (!rc) rc = copy_d2d(a, a->segE, a->E, 3 * N);
    if (!rc) rc = copy_d2d(a, a->recH, a->H, 3 * N);
    if (!rc) rc = copy_d2d(a, a->segPhiE, a->phiE, PL);
    if (!rc) rc = copy_d2d(a, a->recPhiH, a->phiH, PL);
    if (rc) return rc;
    const PhiSet recPH = phiset(a, a->recPhiH);
    for (int it = last0; it < T; ++it) {
      const int m = it - last0;
      float* Em = a->segE + (size_t)m * 3 * N;
      float* Hm = a->segH + (size_t)m * 3 * N;
      const float* Hprev = m == 0 ? a->recH : a->segH + (size_t)(m - 1) * 3 * N;
      adj_fwd_rx<<<1, 64, 0, a->stream>>>(a->p, Em, traces, it);
      adj_fwd_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, Em, Hprev, Hm, recPH);
      adj_fwd_e<<<a->grid, kAdjThreads, 0, a->stream>>>(
          a->p, Em, a->segE + (size_t)(m + 1) * 3 * N, Hm, phiset(a, a->segPhiE + (size_t)m * PL),
          phiset(a, a->segPhiE + (size_t)(m + 1) * PL), it);
    }
  }
  AK(cudaGetLastError());
  AK(cudaStreamSynchronize(a->stream));
  a->forward_done = true;
  a->resident = true;
  return GBF_OK;
}

int gbf_adj_backward(gbf_adj* a, const float* CA, const float* CB, const float* gtraces,
                     double* gCA, double* gCB) {
  if (!a || !CA || !CB || !gtraces || !gCA || !gCB) return GBF_EINVAL;
  if (!a->forward_done) return afail(a, GBF_ESTATE, "gbf_adj_backward: run gbf_adj_forward first");
  const size_t N = a->N, PL = a->phi_len, ck = 6 * N + 2 * PL;
  const int T = a->d.iterations;
  a->p.CA = CA;
  a->p.CB = CB;
  for (float* z : {a->lE, a->lH, a->uE, a->uH})
    AK(cudaMemsetAsync(z, 0, sizeof(float) * 3 * N, a->stream));
  if (PL)
    for (float* z : {a->lphiE, a->lphiH, a->dFE, a->dFH})
      AK(cudaMemsetAsync(z, 0, sizeof(float) * PL, a->stream));
  AK(cudaMemsetAsync(gCA, 0, sizeof(double) * 3 * N, a->stream));
  AK(cudaMemsetAsync(gCB, 0, sizeof(double) * 3 * N, a->stream));
  AdjStep b;
  b.lE = a->lE; b.lH = a->lH; b.uE = a->uE; b.uH = a->uH;
  b.lphiE = phiset(a, a->lphiE);
  b.lphiH = phiset(a, a->lphiH);
  b.dFE = phiset(a, a->dFE);
  b.dFH = phiset(a, a->dFH);
  b.gCA = a->gCA;
  b.gCB = a->gCB;
  b.gtr = gtraces;
  const PhiSet recPH = phiset(a, a->recPhiH);
  const int fold_blocks = a->grid;
  // the fp32 partials add up at most `span` steps (ceil(sqrt(T))) before they go into fp64,
  // however long a segment is
  int span = 1;
  while ((long long)span * span < T) ++span;
  for (int c = a->nck - 1; c >= 0; --c) {
    const int n0 = a->seg[c];
    const int n1 = a->seg[c + 1];
    const float* src = a->ckpt + (size_t)c * ck;
    const bool have = a->resident && c == a->nck - 1;   // left in the slots by the forward
    a->resident = false;
    int rc = have ? 0 : copy_d2d(a, a->segE, src, 3 * N);
    if (!rc && !have) rc = copy_d2d(a, a->recH, src + 3 * N, 3 * N);
    if (!rc && !have) rc = copy_d2d(a, a->segPhiE, src + 6 * N, PL);
    if (!rc && !have) rc = copy_d2d(a, a->recPhiH, src + 6 * N + PL, PL);
    if (rc) return rc;
    // recompute the segment into its slots: E_m, PhiE_m (m = 0..K) and H^{m+1/2} (m = 0..K-1)
    for (int it = have ? n1 : n0; it < n1; ++it) {
      const int m = it - n0;
      float* Em = a->segE + (size_t)m * 3 * N;
      float* Hm = a->segH + (size_t)m * 3 * N;
      const float* Hprev = m == 0 ? a->recH : a->segH + (size_t)(m - 1) * 3 * N;
      adj_fwd_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, Em, Hprev, Hm, recPH);
      adj_fwd_e<<<a->grid, kAdjThreads, 0, a->stream>>>(
          a->p, Em, a->segE + (size_t)(m + 1) * 3 * N, Hm, phiset(a, a->segPhiE + (size_t)m * PL),
          phiset(a, a->segPhiE + (size_t)(m + 1) * PL), it);
    }
    AK(cudaMemsetAsync(a->gCA, 0, sizeof(float) * 3 * N, a->stream));
    AK(cudaMemsetAsync(a->gCB, 0, sizeof(float) * 3 * N, a->stream));
    // undo the segment's steps in reverse
    int since = 0;
    for (int it = n1 - 1; it >= n0; --it) {
      const int m = it - n0;
      b.En = a->segE + (size_t)m * 3 * N;
      b.Hh = a->segH + (size_t)m * 3 * N;
      b.PEn = phiset(a, a->segPhiE + (size_t)m * PL);
      b.it = it;
      b.finish = it + 1 < T ? 1 : 0;
      adj_e_step<<<a->grid_be, kAdjThreads, 0, a->stream>>>(a->p, b);
      adj_h_step<<<a->grid_bh, kAdjThreads, 0, a->stream>>>(a->p, b);
      if (++since == span || it == n0) {
        adj_fold<<<fold_blocks, kAdjThreads, 0, a->stream>>>(a->gCA, gCA, 3 * (long long)N);
        adj_fold<<<fold_blocks, kAdjThreads, 0, a->stream>>>(a->gCB, gCB, 3 * (long long)N);
        since = 0;
      }
    }
    AK(cudaGetLastError());
  }
  AK(cudaStreamSynchronize(a->stream));
  return GBF_OK;
}

// Fixed device scratch of gbf_adj_backward_static: the fp32 per-segment partial sums of the
// two gradients (3N floats each), which gbf_adj_backward keeps in buffers of the context (those
// are still allocated by gbf_adj_create; the static call only keeps its partials here instead).
// 16 MiB, enough for grids of up to kStaticScratchFloats / 6 = 699,050 nodes per component;
// every device that loads the library holds it, whether or not the call is used.
constexpr size_t kStaticScratchFloats = (size_t)4 << 20;
static __device__ __align__(256) float g_static_scratch[kStaticScratchFloats];
constexpr int kStaticMaxDevices = 64;
static float* g_static_scratch_addr[kStaticMaxDevices];
static std::mutex g_static_scratch_lock;

int gbf_adj_backward_static(gbf_adj* a, const float* CA, const float* CB, const float* gtraces,
                            double* gCA, double* gCB) {
  if (!a || !CA || !CB || !gtraces || !gCA || !gCB) return GBF_EINVAL;
  const size_t need = 6 * (size_t)a->N;
  if (need > kStaticScratchFloats)
    return afail(a, GBF_EINVAL,
                 "gbf_adj_backward_static: the grid has %lld nodes per component; the fixed "
                 "scratch holds the partial sums of at most %zu (use gbf_adj_backward)",
                 a->N, kStaticScratchFloats / 6);
  if (a->device < 0 || a->device >= kStaticMaxDevices)
    return afail(a, GBF_EINVAL, "gbf_adj_backward_static: device %d is beyond the %d supported",
                 a->device, kStaticMaxDevices);
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != a->device)
    return afail(a, GBF_ESTATE, "gbf_adj_backward_static: call with the context's device (%d) current",
                 a->device);
  float* base = nullptr;
  {
    std::lock_guard<std::mutex> g(g_static_scratch_lock);
    base = g_static_scratch_addr[a->device];
    if (base) {
      // a device reset since the address was taken unloads the module and the array with it:
      // the cached address must still name device memory of this device, else it is taken anew
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, base) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
          at.device != a->device) {
        (void)cudaGetLastError();
        base = nullptr;
        g_static_scratch_addr[a->device] = nullptr;
      }
    }
    if (!base) {
      // once per device: the address of the array in this device's copy of the module
      void* addr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&addr, g_static_scratch);
      if (e != cudaSuccess)
        return afail(a, GBF_ECUDA, "gbf_adj_backward_static: scratch address: %s",
                     cudaGetErrorString(e));
      base = static_cast<float*>(addr);
      g_static_scratch_addr[a->device] = base;
    }
  }
  // gbf_adj_backward zeroes the partials before each segment, so the scratch needs no
  // particular contents on entry; only the two pointers are swapped for this call.
  float* keepA = a->gCA;
  float* keepB = a->gCB;
  a->gCA = base;
  a->gCB = base + 3 * (size_t)a->N;
  const int rc = gbf_adj_backward(a, CA, CB, gtraces, gCA, gCB);
  // on failure, work already queued may still use the array: wait for it, so that a return
  // means the call is done with the array on every path
  if (rc != GBF_OK) (void)cudaStreamSynchronize(a->stream);
  a->gCA = keepA;
  a->gCB = keepB;
  return rc;
}

}  // extern "C"
