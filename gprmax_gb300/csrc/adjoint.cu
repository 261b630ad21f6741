// adjoint.cu — differentiable time loop: forward kernels with per-edge E coefficients and the
// discrete adjoint (transposed updates, reverse time) with checkpoint-and-recompute.
//
// Model (gprmax_gb300/adjoint.py states it in full): the reference's Yee update
// (fields_updates_ext.pyx update_electric/update_magnetic), HORIPML order-1 slab corrections
// (pml_updates_{electric,magnetic}_HORIPML_ext.pyx order1_*), Hertzian dipoles
// (sources.py:163-193) and field receivers (fields_outputs.py:40-67), with one (CA, CB) pair per
// E edge instead of a material-ID lookup, free-space H coefficients and cubic cells. Phi state
// lives in full-grid arrays (one per slab axis and tangential component); only slab nodes use
// them.
//
// Adjoint of one iteration s_n -> s_{n+1} (H half-step, then E half-step and sources), given the
// adjoint lambda of s_{n+1} and the forward E_n, H^{n+1/2}, PhiE_n of the segment being undone:
//   adj_e_nodes   per E node: u = CB/d * lamE, lamE <- CA * lamE, PML: the Phi and dF adjoints,
//                 gradients dL/dCA += lamE * E_n, dL/dCB += lamE * (curl/d, PML X, source)
//   adj_e_to_h    per H node: lamH += transposed E curl of u, transposed PML differences
//   adj_h_nodes   per H node: u = DB/d * lamH, PML Phi and dF adjoints
//   adj_h_to_e    per E node: lamE += transposed H curl of u, transposed PML differences
//   adj_receivers lamE at receivers += dL/d(trace sample n)
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbfdtd.h"
#define GBF_KERNELS_ONLY
#include "fdtd_kernels.cuh"

using namespace gbf;

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjSrcMax = 16;

struct AdjParams {
  int nx, ny, nz, sx, sy, ncomp;
  float rd;      // 1 / d
  float dbd;     // H curl coefficient DB / d
  float srcm;    // H PML coefficient DB
  int T[6];      // slab thickness, x0 y0 z0 xmax ymax zmax
  const float* R[6];  // per slab [8][T]: ERA ERB ERE ERF HRA HRB HRE HRF (CFS term 0)
  float* E;      // [3][ncomp] working state
  float* H;
  float* phiE;   // [6][ncomp]: pairs x:(Ey,Ez) y:(Ex,Ez) z:(Ex,Ey)
  float* phiH;   // [6][ncomp]: pairs x:(Hy,Hz) y:(Hx,Hz) z:(Hx,Hy)
  const float* CA;   // [3][ncomp]
  const float* CB;
  int nsrc;
  int src_comp[kAdjSrcMax], src_idx[kAdjSrcMax];
  float src_scale[kAdjSrcMax];
  const float* waves;    // [nsrc][iterations]
  int iterations;
  int nrx;
  const int* rx;         // [nrx][2]: component, node index
};

struct AdjBuffers {
  float* lE;     // [3][ncomp] adjoint of E
  float* lH;
  float* lphiE;  // [6][ncomp]
  float* lphiH;
  float* uE;     // [3][ncomp] CB/d * lamE on updated edges
  float* uH;
  float* dFE;    // [6][ncomp] adjoint of the PML differences
  float* dFH;
  const float* En;    // forward E_n        [3][ncomp]
  const float* Hh;    // forward H^{n+1/2}  [3][ncomp]
  const float* PEn;   // forward PhiE_n     [6][ncomp]
  double* gCA;        // [3][ncomp]
  double* gCB;
};

struct Node {
  int i, j, k, idx;
};

__device__ __forceinline__ Node node_of(int q, const AdjParams& p) {
  Node n;
  n.i = q / p.sx;
  const int r = q - n.i * p.sx;
  n.j = r / p.sy;
  n.k = r - n.j * p.sy;
  n.idx = q;
  return n;
}

// pair index and sign of slab axis AX for field component C (electric or magnetic); -1 if C is
// not tangential to AX. E: x (Ey -, Ez +), y (Ex +, Ez -), z (Ex -, Ey +); H opposite signs.
__host__ __device__ constexpr int pair_of(int AX, int C) {
  return AX == 0 ? (C == 1 ? 0 : C == 2 ? 1 : -1)
       : AX == 1 ? (C == 0 ? 2 : C == 2 ? 3 : -1)
                 : (C == 0 ? 4 : C == 1 ? 5 : -1);
}
__host__ __device__ constexpr float pair_sign(bool electric, int AX, int C) {
  return (electric != ((AX == 0) ? (C == 1) : (AX == 1) ? (C == 2) : (C == 0))) ? 1.f : -1.f;
}
// the component whose difference drives the pair (E pairs use H, H pairs use E)
__host__ __device__ constexpr int pair_driver(int AX, int C) {
  return AX == 0 ? (C == 1 ? 2 : 1) : AX == 1 ? (C == 0 ? 2 : 0) : (C == 0 ? 1 : 0);
}

__device__ __forceinline__ int axis_stride(int AX, const AdjParams& p) {
  return AX == 0 ? p.sx : AX == 1 ? p.sy : 1;
}

// slab membership along an axis (0 out, 1 minus, 2 plus) and the profile index
template <bool ELECTRIC>
__device__ __forceinline__ int member(int c, int n, int Tm, int Tp, int& pr) {
  return axis_member<ELECTRIC>(c, n, Tm, Tp, pr);
}

__device__ __forceinline__ const float* slab_rows(const AdjParams& p, int AX, int where, int& T) {
  const int s = AX + (where == 2 ? 3 : 0);
  T = p.T[s];
  return p.R[s];
}

// E node inside the E domain and in the slab of axis AX? (E ranges)
__device__ __forceinline__ bool e_in_slab(const AdjParams& p, int AX, int i, int j, int k,
                                          int& where, int& pr) {
  if (i < 0 || j < 0 || k < 0 || i >= p.nx || j >= p.ny || k >= p.nz) return false;
  const int c = AX == 0 ? i : AX == 1 ? j : k;
  const int n = AX == 0 ? p.nx : AX == 1 ? p.ny : p.nz;
  where = member<true>(c, n, p.T[AX], p.T[AX + 3], pr);
  return where != 0;
}

// H node inside the H PML domain (all coordinates < n) and in the slab of axis AX? (H ranges)
__device__ __forceinline__ bool h_in_slab(const AdjParams& p, int AX, int i, int j, int k,
                                          int& where, int& pr) {
  if (i < 0 || j < 0 || k < 0 || i >= p.nx || j >= p.ny || k >= p.nz) return false;
  const int c = AX == 0 ? i : AX == 1 ? j : k;
  const int n = AX == 0 ? p.nx : AX == 1 ? p.ny : p.nz;
  where = member<false>(c, n, p.T[AX], p.T[AX + 3], pr);
  return where != 0;
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

// E curl term of component C at idx from H (the bracket multiplied by CB/d)
__device__ __forceinline__ float e_curl(int C, int idx, const float* H, const AdjParams& p) {
  const float* Hx = H;
  const float* Hy = H + p.ncomp;
  const float* Hz = H + 2 * (size_t)p.ncomp;
  if (C == 0) return (Hz[idx] - Hz[idx - p.sy]) - (Hy[idx] - Hy[idx - 1]);
  if (C == 1) return (Hx[idx] - Hx[idx - 1]) - (Hz[idx] - Hz[idx - p.sx]);
  return (Hy[idx] - Hy[idx - p.sx]) - (Hx[idx] - Hx[idx - p.sy]);
}

// Apply the slab corrections of component C in the reference's slab order (x0 y0 z0 xmax ymax
// zmax): with one slab per axis, axis b comes before a (a < b) only when a is on its plus side
// and b on its minus side.
template <int C>
__device__ __forceinline__ float apply_terms(float F, const int* where, const float* t) {
  constexpr int a = C == 0 ? 1 : 0;
  constexpr int b = C == 2 ? 1 : 2;
  if (where[a] && where[b] && where[a] == 2 && where[b] == 1) {
    F = F + t[b];
    F = F + t[a];
  } else {
    if (where[a]) F = F + t[a];
    if (where[b]) F = F + t[b];
  }
  return F;
}

// ---- forward --------------------------------------------------------------------------
__global__ void __launch_bounds__(kAdjThreads) adj_fwd_h(const __grid_constant__ AdjParams p) {
  const int stride = gridDim.x * blockDim.x;
  const float* Ex = p.E;
  const float* Ey = p.E + p.ncomp;
  const float* Ez = p.E + 2 * (size_t)p.ncomp;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int idx = n.idx;
    float h[3];
    for (int C = 0; C < 3; ++C) h[C] = p.H[C * (size_t)p.ncomp + idx];
    if (h_updated(0, n.i, n.j, n.k, p))
      h[0] = h[0] - p.dbd * (Ez[idx + p.sy] - Ez[idx]) + p.dbd * (Ey[idx + 1] - Ey[idx]);
    if (h_updated(1, n.i, n.j, n.k, p))
      h[1] = h[1] - p.dbd * (Ex[idx + 1] - Ex[idx]) + p.dbd * (Ez[idx + p.sx] - Ez[idx]);
    if (h_updated(2, n.i, n.j, n.k, p))
      h[2] = h[2] - p.dbd * (Ey[idx + p.sx] - Ey[idx]) + p.dbd * (Ex[idx + p.sy] - Ex[idx]);
    int where[3] = {0, 0, 0};
    float t[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // [component][axis]
    bool any = false;
#pragma unroll
    for (int AX = 0; AX < 3; ++AX) {
      int pr = 0;
      if (!h_in_slab(p, AX, n.i, n.j, n.k, where[AX], pr)) { where[AX] = 0; continue; }
      any = true;
      int T;
      const float* R = slab_rows(p, AX, where[AX], T);
      const float RA = R[4 * T + pr], RB = R[5 * T + pr], RE = R[6 * T + pr], RF = R[7 * T + pr];
      const int st = axis_stride(AX, p);
#pragma unroll
      for (int C = 0; C < 3; ++C) {
        const int q2 = pair_of(AX, C);
        if (q2 < 0) continue;
        const float* D = p.E + pair_driver(AX, C) * (size_t)p.ncomp;
        const float dF = (D[idx + st] - D[idx]) * p.rd;
        float* phi = p.phiH + q2 * (size_t)p.ncomp + idx;
        const float ph = *phi;
        const float X = (RA - 1.0f) * dF + RB * ph;
        *phi = RE * ph - RF * dF;
        t[C][AX] = pair_sign(false, AX, C) * (p.srcm * X);
      }
    }
    if (any) {
      h[0] = apply_terms<0>(h[0], where, t[0]);
      h[1] = apply_terms<1>(h[1], where, t[1]);
      h[2] = apply_terms<2>(h[2], where, t[2]);
    }
    for (int C = 0; C < 3; ++C) p.H[C * (size_t)p.ncomp + idx] = h[C];
  }
}

__global__ void __launch_bounds__(kAdjThreads) adj_fwd_e(const __grid_constant__ AdjParams p, int it) {
  const int stride = gridDim.x * blockDim.x;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int idx = n.idx;
    float e[3], cb[3];
    for (int C = 0; C < 3; ++C) {
      e[C] = p.E[C * (size_t)p.ncomp + idx];
      cb[C] = p.CB[C * (size_t)p.ncomp + idx];
      if (e_updated(C, n.i, n.j, n.k, p))
        e[C] = p.CA[C * (size_t)p.ncomp + idx] * e[C] + (cb[C] * p.rd) * e_curl(C, idx, p.H, p);
    }
    int where[3] = {0, 0, 0};
    float t[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    bool any = false;
#pragma unroll
    for (int AX = 0; AX < 3; ++AX) {
      int pr = 0;
      if (!e_in_slab(p, AX, n.i, n.j, n.k, where[AX], pr)) { where[AX] = 0; continue; }
      any = true;
      int T;
      const float* R = slab_rows(p, AX, where[AX], T);
      const float RA = R[pr], RB = R[T + pr], RE = R[2 * T + pr], RF = R[3 * T + pr];
      const int st = axis_stride(AX, p);
#pragma unroll
      for (int C = 0; C < 3; ++C) {
        const int q2 = pair_of(AX, C);
        if (q2 < 0) continue;
        const float* D = p.H + pair_driver(AX, C) * (size_t)p.ncomp;
        const float dF = (D[idx] - D[idx - st]) * p.rd;
        float* phi = p.phiE + q2 * (size_t)p.ncomp + idx;
        const float ph = *phi;
        const float X = (RA - 1.0f) * dF + RB * ph;
        *phi = RE * ph - RF * dF;
        t[C][AX] = pair_sign(true, AX, C) * (cb[C] * X);
      }
    }
    if (any) {
      e[0] = apply_terms<0>(e[0], where, t[0]);
      e[1] = apply_terms<1>(e[1], where, t[1]);
      e[2] = apply_terms<2>(e[2], where, t[2]);
    }
    for (int s = 0; s < p.nsrc; ++s)
      if (p.src_idx[s] == idx) {
        const int C = p.src_comp[s];
        e[C] = e[C] - cb[C] * p.waves[(size_t)s * p.iterations + it] * p.src_scale[s];
      }
    for (int C = 0; C < 3; ++C) p.E[C * (size_t)p.ncomp + idx] = e[C];
  }
}

__global__ void adj_fwd_rx(const __grid_constant__ AdjParams p, float* traces, int it) {
  for (int r = threadIdx.x; r < p.nrx; r += blockDim.x) {
    const int C = p.rx[2 * r], idx = p.rx[2 * r + 1];
    traces[(size_t)r * p.iterations + it] = p.E[C * (size_t)p.ncomp + idx];
  }
}

// ---- adjoint --------------------------------------------------------------------------
__global__ void __launch_bounds__(kAdjThreads)
adj_e_nodes(const __grid_constant__ AdjParams p, const __grid_constant__ AdjBuffers b, int it) {
  const int stride = gridDim.x * blockDim.x;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int idx = n.idx;
    float lam[3], cb[3];
    double gcb[3] = {0.0, 0.0, 0.0};
    for (int C = 0; C < 3; ++C) {
      const size_t o = C * (size_t)p.ncomp + idx;
      lam[C] = b.lE[o];
      cb[C] = p.CB[o];
      float u = 0.f, lnew = lam[C];
      if (e_updated(C, n.i, n.j, n.k, p)) {
        u = (cb[C] * p.rd) * lam[C];
        lnew = p.CA[o] * lam[C];
        b.gCA[o] += (double)lam[C] * (double)b.En[o];
        gcb[C] += (double)lam[C] * (double)(p.rd * e_curl(C, idx, b.Hh, p));
      }
      b.uE[o] = u;
      b.lE[o] = lnew;
    }
#pragma unroll
    for (int AX = 0; AX < 3; ++AX) {
      int where = 0, pr = 0;
      if (!e_in_slab(p, AX, n.i, n.j, n.k, where, pr)) continue;
      int T;
      const float* R = slab_rows(p, AX, where, T);
      const float RA = R[pr], RB = R[T + pr], RE = R[2 * T + pr], RF = R[3 * T + pr];
      const int st = axis_stride(AX, p);
#pragma unroll
      for (int C = 0; C < 3; ++C) {
        const int q2 = pair_of(AX, C);
        if (q2 < 0) continue;
        const size_t o = q2 * (size_t)p.ncomp + idx;
        const float s = pair_sign(true, AX, C);
        const float Xb = s * cb[C] * lam[C];
        const float lph = b.lphiE[o];
        b.dFE[o] = (RA - 1.0f) * Xb - RF * lph;
        b.lphiE[o] = RB * Xb + RE * lph;
        const float* D = b.Hh + pair_driver(AX, C) * (size_t)p.ncomp;
        const float dF = (D[idx] - D[idx - st]) * p.rd;
        const float X = (RA - 1.0f) * dF + RB * b.PEn[o];
        gcb[C] += (double)s * (double)X * (double)lam[C];
      }
    }
    for (int s = 0; s < p.nsrc; ++s)
      if (p.src_idx[s] == idx) {
        const int C = p.src_comp[s];
        gcb[C] -= (double)p.waves[(size_t)s * p.iterations + it] * (double)p.src_scale[s] *
                  (double)lam[C];
      }
    for (int C = 0; C < 3; ++C) b.gCB[C * (size_t)p.ncomp + idx] += gcb[C];
  }
}

// u of E component C at node (i, j, k), 0 outside the arrays
__device__ __forceinline__ float u_at(const float* u, int C, int i, int j, int k,
                                      const AdjParams& p) {
  if (i < 0 || j < 0 || k < 0 || i > p.nx || j > p.ny || k > p.nz) return 0.f;
  return u[C * (size_t)p.ncomp + i * p.sx + j * p.sy + k];
}

// adjoint of the PML difference of pair (AX, C) at E node (i, j, k), 0 off the slab
__device__ __forceinline__ float dFE_at(const AdjBuffers& b, const AdjParams& p, int AX, int C,
                                        int i, int j, int k) {
  int where, pr;
  if (!e_in_slab(p, AX, i, j, k, where, pr)) return 0.f;
  return b.dFE[pair_of(AX, C) * (size_t)p.ncomp + i * p.sx + j * p.sy + k];
}

__device__ __forceinline__ float dFH_at(const AdjBuffers& b, const AdjParams& p, int AX, int C,
                                        int i, int j, int k) {
  int where, pr;
  if (!h_in_slab(p, AX, i, j, k, where, pr)) return 0.f;
  return b.dFH[pair_of(AX, C) * (size_t)p.ncomp + i * p.sx + j * p.sy + k];
}

__global__ void __launch_bounds__(kAdjThreads)
adj_e_to_h(const __grid_constant__ AdjParams p, const __grid_constant__ AdjBuffers b) {
  const int stride = gridDim.x * blockDim.x;
  const float* u = b.uE;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int i = n.i, j = n.j, k = n.k;
    // transposed E curl (E update: Ex += u-terms of Hz(j), Hz(j-1), Hy(k), Hy(k-1) ...)
    float gx = u_at(u, 1, i, j, k, p) - u_at(u, 1, i, j, k + 1, p) - u_at(u, 2, i, j, k, p) +
               u_at(u, 2, i, j + 1, k, p);
    float gy = -u_at(u, 0, i, j, k, p) + u_at(u, 0, i, j, k + 1, p) + u_at(u, 2, i, j, k, p) -
               u_at(u, 2, i + 1, j, k, p);
    float gz = u_at(u, 0, i, j, k, p) - u_at(u, 0, i, j + 1, k, p) - u_at(u, 1, i, j, k, p) +
               u_at(u, 1, i + 1, j, k, p);
    // transposed PML differences: dF(e) = (H(e) - H(e - a)) / d feeds H at e and e - a
    const float rd = p.rd;
    gz += rd * (dFE_at(b, p, 0, 1, i, j, k) - dFE_at(b, p, 0, 1, i + 1, j, k) +
                dFE_at(b, p, 1, 0, i, j, k) - dFE_at(b, p, 1, 0, i, j + 1, k));
    gy += rd * (dFE_at(b, p, 0, 2, i, j, k) - dFE_at(b, p, 0, 2, i + 1, j, k) +
                dFE_at(b, p, 2, 0, i, j, k) - dFE_at(b, p, 2, 0, i, j, k + 1));
    gx += rd * (dFE_at(b, p, 1, 2, i, j, k) - dFE_at(b, p, 1, 2, i, j + 1, k) +
                dFE_at(b, p, 2, 1, i, j, k) - dFE_at(b, p, 2, 1, i, j, k + 1));
    b.lH[n.idx] += gx;
    b.lH[p.ncomp + (size_t)n.idx] += gy;
    b.lH[2 * (size_t)p.ncomp + n.idx] += gz;
  }
}

__global__ void __launch_bounds__(kAdjThreads)
adj_h_nodes(const __grid_constant__ AdjParams p, const __grid_constant__ AdjBuffers b) {
  const int stride = gridDim.x * blockDim.x;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int idx = n.idx;
    float lam[3];
    for (int C = 0; C < 3; ++C) {
      const size_t o = C * (size_t)p.ncomp + idx;
      lam[C] = b.lH[o];
      b.uH[o] = h_updated(C, n.i, n.j, n.k, p) ? p.dbd * lam[C] : 0.f;
    }
#pragma unroll
    for (int AX = 0; AX < 3; ++AX) {
      int where = 0, pr = 0;
      if (!h_in_slab(p, AX, n.i, n.j, n.k, where, pr)) continue;
      int T;
      const float* R = slab_rows(p, AX, where, T);
      const float RA = R[4 * T + pr], RB = R[5 * T + pr], RE = R[6 * T + pr], RF = R[7 * T + pr];
#pragma unroll
      for (int C = 0; C < 3; ++C) {
        const int q2 = pair_of(AX, C);
        if (q2 < 0) continue;
        const size_t o = q2 * (size_t)p.ncomp + idx;
        const float Xb = pair_sign(false, AX, C) * p.srcm * lam[C];
        const float lph = b.lphiH[o];
        b.dFH[o] = (RA - 1.0f) * Xb - RF * lph;
        b.lphiH[o] = RB * Xb + RE * lph;
      }
    }
  }
}

__global__ void __launch_bounds__(kAdjThreads)
adj_h_to_e(const __grid_constant__ AdjParams p, const __grid_constant__ AdjBuffers b) {
  const int stride = gridDim.x * blockDim.x;
  const float* u = b.uH;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < p.ncomp; q += stride) {
    const Node n = node_of(q, p);
    const int i = n.i, j = n.j, k = n.k;
    // transposed H curl (Hx -= DB/d (Ez(j+1) - Ez) - DB/d (Ey(k+1) - Ey) ...)
    float gx = u_at(u, 1, i, j, k, p) - u_at(u, 1, i, j, k - 1, p) + u_at(u, 2, i, j - 1, k, p) -
               u_at(u, 2, i, j, k, p);
    float gy = u_at(u, 0, i, j, k - 1, p) - u_at(u, 0, i, j, k, p) - u_at(u, 2, i - 1, j, k, p) +
               u_at(u, 2, i, j, k, p);
    float gz = -u_at(u, 0, i, j - 1, k, p) + u_at(u, 0, i, j, k, p) + u_at(u, 1, i - 1, j, k, p) -
               u_at(u, 1, i, j, k, p);
    // transposed PML differences: dF(h) = (E(h + a) - E(h)) / d feeds E at h + a and h
    const float rd = p.rd;
    gz += rd * (dFH_at(b, p, 0, 1, i - 1, j, k) - dFH_at(b, p, 0, 1, i, j, k) +
                dFH_at(b, p, 1, 0, i, j - 1, k) - dFH_at(b, p, 1, 0, i, j, k));
    gy += rd * (dFH_at(b, p, 0, 2, i - 1, j, k) - dFH_at(b, p, 0, 2, i, j, k) +
                dFH_at(b, p, 2, 0, i, j, k - 1) - dFH_at(b, p, 2, 0, i, j, k));
    gx += rd * (dFH_at(b, p, 1, 2, i, j - 1, k) - dFH_at(b, p, 1, 2, i, j, k) +
                dFH_at(b, p, 2, 1, i, j, k - 1) - dFH_at(b, p, 2, 1, i, j, k));
    b.lE[n.idx] += gx;
    b.lE[p.ncomp + (size_t)n.idx] += gy;
    b.lE[2 * (size_t)p.ncomp + n.idx] += gz;
  }
}

__global__ void adj_receivers(const __grid_constant__ AdjParams p, AdjBuffers b,
                              const float* gtraces, int it) {
  if (threadIdx.x != 0) return;
  for (int r = 0; r < p.nrx; ++r) {
    const int C = p.rx[2 * r], idx = p.rx[2 * r + 1];
    b.lE[C * (size_t)p.ncomp + idx] += gtraces[(size_t)r * p.iterations + it];
  }
}

}  // namespace

// ---- host side -------------------------------------------------------------------------
struct gbf_adj {
  gbf_adj_desc d;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long ncomp = 0;
  int K = 1;                 // checkpoint interval (steps)
  int nck = 0;               // checkpoints
  AdjParams p{};
  std::vector<void*> allocs;
  float* state = nullptr;    // working E, H, phiE, phiH: 18 * ncomp
  float* ckpt = nullptr;     // nck * 18 * ncomp
  float* seg = nullptr;      // K * 12 * ncomp: E_n, H^{n+1/2}, PhiE_n of each step of a segment
  float* adj = nullptr;      // lE lH (3 each) lphiE lphiH (6 each) uE uH (3 each) dFE dFH (6 each)
  float* pml_rows = nullptr; // 6 * 8 * Tmax
  float* waves = nullptr;
  int* rx = nullptr;
  bool forward_done = false;
  int grid = 0;
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

static int adj_alloc(gbf_adj* a, void** ptr, size_t bytes) {
  AK(cudaMalloc(ptr, bytes));
  a->allocs.push_back(*ptr);
  AK(cudaMemsetAsync(*ptr, 0, bytes, a->stream));
  return GBF_OK;
}

static void set_state_ptrs(gbf_adj* a) {
  const size_t N = a->ncomp;
  a->p.E = a->state;
  a->p.H = a->state + 3 * N;
  a->p.phiE = a->state + 6 * N;
  a->p.phiH = a->state + 12 * N;
}

static AdjBuffers buffers(gbf_adj* a, int step_in_seg, double* gCA, double* gCB) {
  const size_t N = a->ncomp;
  AdjBuffers b;
  float* q = a->adj;
  b.lE = q; q += 3 * N;
  b.lH = q; q += 3 * N;
  b.lphiE = q; q += 6 * N;
  b.lphiH = q; q += 6 * N;
  b.uE = q; q += 3 * N;
  b.uH = q; q += 3 * N;
  b.dFE = q; q += 6 * N;
  b.dFH = q;
  const float* s = a->seg + (size_t)step_in_seg * 12 * N;
  b.En = s;
  b.Hh = s + 3 * N;
  b.PEn = s + 6 * N;
  b.gCA = gCA;
  b.gCB = gCB;
  return b;
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
  if (d.nsrc < 0 || d.nsrc > kAdjSrcMax || d.nrx < 1)
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: 0..%d sources and at least one receiver", kAdjSrcMax);
  if (d.reserved[0] || d.reserved[1] || d.reserved[2])
    return afail(nullptr, GBF_EINVAL, "gbf_adj_create: reserved fields must be zero");
  const int n3[3] = {d.nx, d.ny, d.nz};
  for (int s = 0; s < 6; ++s)
    if (d.pml_thickness[s] < 0 || 2 * d.pml_thickness[s] >= n3[s % 3])
      return afail(nullptr, GBF_EINVAL, "gbf_adj_create: PML slab %d thickness %d too large", s, d.pml_thickness[s]);
  const long long N = (long long)(d.nx + 1) * (d.ny + 1) * (d.nz + 1);
  if (N > (1LL << 31) - 1) return afail(nullptr, GBF_EINVAL, "gbf_adj_create: more than 2^31 nodes");
  gbf_adj* a = new gbf_adj();
  a->d = d;
  a->ncomp = N;
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
  int Tmax = 1;
  for (int s = 0; s < 6; ++s) Tmax = d.pml_thickness[s] > Tmax ? d.pml_thickness[s] : Tmax;
  int rc = GBF_OK;
  auto A = [&](void** ptr, size_t bytes) { if (rc == GBF_OK) rc = adj_alloc(a, ptr, bytes); };
  A((void**)&a->state, sizeof(float) * 18 * (size_t)N);
  A((void**)&a->ckpt, sizeof(float) * 18 * (size_t)N * a->nck);
  A((void**)&a->seg, sizeof(float) * 12 * (size_t)N * a->K);
  A((void**)&a->adj, sizeof(float) * 36 * (size_t)N);
  A((void**)&a->pml_rows, sizeof(float) * 6 * 8 * Tmax);
  A((void**)&a->waves, sizeof(float) * (size_t)(d.nsrc + 1) * d.iterations);
  A((void**)&a->rx, sizeof(int) * 2 * d.nrx);
  if (rc != GBF_OK) {
    g_adj_err = a->err;
    gbf_adj_destroy(a);
    return rc;
  }
  AdjParams& p = a->p;
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  p.sy = d.nz + 1;
  p.sx = (d.ny + 1) * (d.nz + 1);
  p.ncomp = (int)N;
  p.rd = 1.0f / d.d;
  p.dbd = d.dbd;
  p.srcm = d.srcm;
  for (int s = 0; s < 6; ++s) {
    p.T[s] = d.pml_thickness[s];
    p.R[s] = a->pml_rows + (size_t)s * 8 * Tmax;
  }
  set_state_ptrs(a);
  p.nsrc = 0;
  p.waves = a->waves;
  p.iterations = d.iterations;
  p.nrx = 0;
  p.rx = a->rx;
  int dev = 0, sms = 1, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, adj_e_nodes, kAdjThreads, 0);
  a->grid = sms * (per > 0 ? per : 1);
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
    AK(cudaMemcpyAsync(const_cast<float*>(a->p.R[slab]) + (size_t)r * T, rows[r], sizeof(float) * T,
                       cudaMemcpyHostToDevice, a->stream));
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
  std::vector<int> rx(2 * d.nrx);
  for (int r = 0; r < d.nrx; ++r) {
    const int C = info[4 * r], i = info[4 * r + 1], j = info[4 * r + 2], k = info[4 * r + 3];
    if (C < 0 || C > 2 || i < 0 || j < 0 || k < 0 || i > d.nx || j > d.ny || k > d.nz)
      return afail(a, GBF_EINVAL, "gbf_adj_set_receivers: receiver %d out of the grid", r);
    rx[2 * r] = C;
    rx[2 * r + 1] = i * a->p.sx + j * a->p.sy + k;
  }
  AK(cudaMemcpyAsync(a->rx, rx.data(), sizeof(int) * rx.size(), cudaMemcpyHostToDevice, a->stream));
  AK(cudaStreamSynchronize(a->stream));
  a->p.nrx = d.nrx;
  return GBF_OK;
}

}  // extern "C"

static void fwd_step(gbf_adj* a, int it, float* traces) {
  if (traces) adj_fwd_rx<<<1, 32, 0, a->stream>>>(a->p, traces, it);
  adj_fwd_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p);
  adj_fwd_e<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, it);
}

extern "C" {

int gbf_adj_forward(gbf_adj* a, const float* CA, const float* CB, float* traces) {
  if (!a || !CA || !CB || !traces) return GBF_EINVAL;
  const size_t N = a->ncomp;
  a->p.CA = CA;
  a->p.CB = CB;
  AK(cudaMemsetAsync(a->state, 0, sizeof(float) * 18 * N, a->stream));
  for (int it = 0; it < a->d.iterations; ++it) {
    if (it % a->K == 0)
      AK(cudaMemcpyAsync(a->ckpt + (size_t)(it / a->K) * 18 * N, a->state, sizeof(float) * 18 * N,
                         cudaMemcpyDeviceToDevice, a->stream));
    fwd_step(a, it, traces);
  }
  AK(cudaGetLastError());
  AK(cudaStreamSynchronize(a->stream));
  a->forward_done = true;
  return GBF_OK;
}

int gbf_adj_backward(gbf_adj* a, const float* CA, const float* CB, const float* gtraces,
                     double* gCA, double* gCB) {
  if (!a || !CA || !CB || !gtraces || !gCA || !gCB) return GBF_EINVAL;
  if (!a->forward_done) return afail(a, GBF_ESTATE, "gbf_adj_backward: run gbf_adj_forward first");
  const size_t N = a->ncomp;
  a->p.CA = CA;
  a->p.CB = CB;
  AK(cudaMemsetAsync(a->adj, 0, sizeof(float) * 36 * N, a->stream));
  AK(cudaMemsetAsync(gCA, 0, sizeof(double) * 3 * N, a->stream));
  AK(cudaMemsetAsync(gCB, 0, sizeof(double) * 3 * N, a->stream));
  const int T = a->d.iterations;
  for (int c = a->nck - 1; c >= 0; --c) {
    const int n0 = c * a->K;
    const int n1 = (n0 + a->K < T) ? n0 + a->K : T;
    // recompute the segment from its checkpoint, keeping what the adjoint steps read
    AK(cudaMemcpyAsync(a->state, a->ckpt + (size_t)c * 18 * N, sizeof(float) * 18 * N,
                       cudaMemcpyDeviceToDevice, a->stream));
    for (int it = n0; it < n1; ++it) {
      float* s = a->seg + (size_t)(it - n0) * 12 * N;
      AK(cudaMemcpyAsync(s, a->p.E, sizeof(float) * 3 * N, cudaMemcpyDeviceToDevice, a->stream));
      AK(cudaMemcpyAsync(s + 6 * N, a->p.phiE, sizeof(float) * 6 * N, cudaMemcpyDeviceToDevice, a->stream));
      adj_fwd_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p);
      AK(cudaMemcpyAsync(s + 3 * N, a->p.H, sizeof(float) * 3 * N, cudaMemcpyDeviceToDevice, a->stream));
      adj_fwd_e<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, it);
    }
    // undo the segment's steps in reverse
    for (int it = n1 - 1; it >= n0; --it) {
      const AdjBuffers b = buffers(a, it - n0, gCA, gCB);
      adj_e_nodes<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, b, it);
      adj_e_to_h<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, b);
      adj_h_nodes<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, b);
      adj_h_to_e<<<a->grid, kAdjThreads, 0, a->stream>>>(a->p, b);
      adj_receivers<<<1, 32, 0, a->stream>>>(a->p, b, gtraces, it);
    }
    AK(cudaGetLastError());
  }
  AK(cudaStreamSynchronize(a->stream));
  return GBF_OK;
}

}  // extern "C"
