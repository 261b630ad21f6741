// fused_step.cuh — one kernel per Yee iteration: the H and E half-steps fused into a single
// pass over the grid, for 3D models without transmission lines whose material IDs pack into
// one word per node (at most 1024 materials).
//
// Per node the arithmetic is exactly that of the two half-step kernels (h_node, e_node in
// fdtd_kernels.cuh: gprMax/fields_updates_ext.pyx:30-412, the pml_updates_* slab corrections in
// slab order, sources, the dispersive A/B update), so results are identical bit for bit. What
// changes is the traffic: E, H, the packed IDs and the dispersive state are read once and E and
// H written once per iteration, instead of E and H being streamed by both half-steps.
//
// Tiling. A block of TJ + 1 warps owns a tile of kTileK (31) consecutive k by TJ consecutive j
// and marches along x over a chunk of planes i0..i1-1. Warp w works on row j = j0 - 1 + w, lane
// l on column k = k0 - 1 + l: warp 0 (the row below the tile) and lane 0 (the node below it in
// k) are halo: their H is formed (the E update of the tile needs H at j-1 and k-1) but neither
// stored nor allowed to advance PML state. At plane i each warp
//   1. publishes its E(i) (Ex, Ez) in shared memory and, after a barrier, takes the j+1 row's
//      from its neighbour warp (the top warp reads that row itself); the k+1 neighbours come
//      from the next lane (warp shuffle; the last lane reads them itself);
//   2. forms H(i) of its row from E(i), E(i+1) and H(i), publishes Hx, Hz, and after a second
//      barrier forms E(i) from H(i) (row j-1 from shared memory, k-1 from the previous lane)
//      and H(i-1) (kept in registers from the previous plane);
//   3. stores E(i), H(i) and the dispersive state of its owned nodes.
// Every global load of plane i + 1 (E of plane i + 2) is issued at the start of plane i, so the
// march streams without waiting on its loads. A chunk starts with one halo plane (H of plane
// i0 - 1, not stored).
//
#pragma once
#include "fdtd_kernels.cuh"

namespace gbf {

constexpr int kTileK = 31;   // k nodes a tile owns (lane 0 is the halo node below them)

// Decomposition of one launch: block b -> k segment b % nseg, j tile (b / nseg) % njt and i
// chunk b / (nseg * njt), the chunk covering planes [ch * L, min((ch + 1) * L, nx + 1)); a block
// has TJ + 1 warps for a tile of TJ rows. nblocks = nseg * njt * nch.
struct FusedTiles {
  int nseg, njt, nch, L, nblocks;
};

constexpr int kFusedMaxPoles = 2;   // models with more poles take the two half-step kernels
typedef void (*FusedFn)(StepParams, FusedTiles);
// per PML kind and tile height (fused_inst.cu, one object each); nullptr when not built
#define GBF_FUSED_DECL(pk, tj) FusedFn fused_kernel_pk##pk##_tj##tj(int np, int uniform_h, int treal);
GBF_FUSED_DECL(0, 7) GBF_FUSED_DECL(1, 7) GBF_FUSED_DECL(2, 7) GBF_FUSED_DECL(3, 7) GBF_FUSED_DECL(4, 7)
GBF_FUSED_DECL(0, 15) GBF_FUSED_DECL(1, 15) GBF_FUSED_DECL(2, 15) GBF_FUSED_DECL(3, 15) GBF_FUSED_DECL(4, 15)
#undef GBF_FUSED_DECL

// Loads of one plane for one node: H, the packed ID words and the dispersive state.
template <int NP, bool TR, int IDPH>
struct PlaneIn {
  float hx, hy, hz;
  uint32_t pe, ph;
  float2 t[3][NP > 0 ? NP : 1];
};

template <int PK, int NP, bool TR, int IDPH, int TJ>
__global__ void __launch_bounds__((TJ + 1) * 32, TJ >= 15 ? 1 : 3)
fused_step(const __grid_constant__ StepParams p, const __grid_constant__ FusedTiles ft) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int NW = TJ + 1;
  // coefficient tables in shared memory: E rows, srce, dispersive records, then H rows, srcm
  extern __shared__ float4 smem_f[];
  __shared__ float2 xE[NW][32];   // E(i) (Ex, Ez) of each warp's row
  __shared__ float2 xH[NW][32];   // new H(i) (Hx, Hz) of each warp's row
  float4* s4;
  float* ss;
  float2* sd;
  e_tables(p, smem_f, s4, ss, sd);
  float4* h4 = reinterpret_cast<float4*>(
      (reinterpret_cast<uintptr_t>(sd + (p.smem ? p.nmat * 3 * p.P : 0)) + 15) & ~(uintptr_t)15);
  float* hs = reinterpret_cast<float*>(h4 + (p.smem ? p.nmat : 0));
  if (p.smem) {
    stage_tables(p, true, s4, ss, NP > 0 ? sd : nullptr);
    if (IDPH) stage_tables(p, false, h4, hs, nullptr);
  }
  const float4* C4 = p.smem ? s4 : p.cE4;
  const float* Cs = p.smem ? ss : p.cEs;
  const float2* CD = (p.smem && NP > 0) ? sd : p.cD;
  HCoef hc;
  hc.C4 = p.smem ? h4 : p.cH4;
  hc.Cs = p.smem ? hs : p.cHs;

  // block -> (k segment, j tile, chunk); warp -> row; lane -> column
  const int b = blockIdx.x;
  const int seg = b % ft.nseg;
  const int rest = b / ft.nseg;
  const int jt = rest % ft.njt;
  const int ch = rest / ft.njt;
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nx = p.nx, ny = p.ny, nz = p.nz, sx = p.sx, sy = p.sy;
  const int k = seg * kTileK - 1 + lane;
  const int j = jt * TJ - 1 + w;
  const bool kv = k >= 0 && k <= nz;           // a node column of the grid
  const bool jv = j >= 0 && j <= ny;           // a node row of the grid
  const bool nodev = kv && jv;
  const bool own = lane > 0 && w > 0 && nodev; // H stored by this thread
  const bool eown = lane > 0 && w > 0 && k < nz && j < ny;   // E formed and stored
  const bool top = w == TJ;                    // reads the j+1 row itself
  const int i0 = ch * ft.L;
  const int i1 = min(i0 + ft.L, nx + 1);
  const int ib = i0 > 0 ? i0 - 1 : 0;          // first plane formed (a halo plane when i0 > 0)
  const int it = (p.nsrcE || p.nsrcH) ? *p.d_it : 0;
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  const float* __restrict__ Hx = p.H[0];
  const float* __restrict__ Hy = p.H[1];
  const float* __restrict__ Hz = p.H[2];
  const int col = j * sy + k;                  // node offset within a plane (when nodev)
  const int colj = (j + 1) * sy + k;           // the j+1 row (top warp, j + 1 <= ny)
  const bool topv = top && kv && j + 1 <= ny;
  const bool k1v = lane == 31 && jv && k + 1 <= nz;

  // sources in this thread's column: bit 0 an E source, bit 1 an H source
  uint32_t smask = 0;
  for (int s = 0; s < p.nsrcE; ++s) {
    const Src& q = p.srcE[s];
    if (q.j == j && q.k == k) smask |= 1u;
  }
  for (int s = 0; s < p.nsrcH; ++s) {
    const Src& q = p.srcH[s];
    if (q.j == j && q.k == k) smask |= 2u;
  }
  // slab membership along z (this column) and y (this row), E and H ranges
  int whEz = 0, prEz = 0, whHz = 0, prHz = 0, whEy = 0, prEy = 0, whHy = 0, prHy = 0;
  if (PK != PML_NONE) {
    whEz = axis_member<true>(k, nz, p.slab[2].T, p.slab[5].T, prEz);
    whHz = axis_member<false>(k, nz, p.slab[2].T, p.slab[5].T, prHz);
    whEy = axis_member<true>(j, ny, p.slab[1].T, p.slab[4].T, prEy);
    whHy = axis_member<false>(j, ny, p.slab[1].T, p.slab[4].T, prHy);
  }

  auto loadE = [&](int pl, float& x, float& y, float& z) {
    const bool v = nodev && pl <= nx;
    const int idx = pl * sx + col;
    x = v ? __ldg(Ex + idx) : 0.f;
    y = v ? __ldg(Ey + idx) : 0.f;
    z = v ? __ldg(Ez + idx) : 0.f;
  };
  // E(pl) at k + 1 (last lane: Ex, Ey) and at j + 1 (top warp: Ex, Ez)
  auto loadEdge = [&](int pl, float& kx, float& ky, float& jx, float& jz) {
    const bool vk = k1v && pl <= nx;
    const bool vj = topv && pl <= nx;
    kx = vk ? __ldg(Ex + pl * sx + col + 1) : 0.f;
    ky = vk ? __ldg(Ey + pl * sx + col + 1) : 0.f;
    jx = vj ? __ldg(Ex + pl * sx + colj) : 0.f;
    jz = vj ? __ldg(Ez + pl * sx + colj) : 0.f;
  };
  auto loadIn = [&](int pl, PlaneIn<NP, TR, IDPH>& q) {
    const bool v = nodev && pl <= nx;
    const int idx = pl * sx + col;
    q.hx = v ? __ldg(Hx + idx) : 0.f;
    q.hy = v ? __ldg(Hy + idx) : 0.f;
    q.hz = v ? __ldg(Hz + idx) : 0.f;
    q.ph = (IDPH && v) ? __ldg(p.PH + idx) : 0u;
    const bool ve = eown && pl < nx && pl >= i0;
    q.pe = ve ? __ldg(p.PE + idx) : 0u;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int qq = 0; qq < NP; ++qq) {
        const long long o = (c * NP + qq) * (long long)p.ncomp + idx;
        q.t[c][qq] = !ve ? make_float2(0.f, 0.f)
                         : (TR ? make_float2(reinterpret_cast<const float*>(p.T)[o], 0.f) : p.T[o]);
      }
  };

  // the pipeline: E of planes i, i + 1 (and i + 2 in flight), the other inputs of plane i (and
  // i + 1 in flight), H of plane i - 1
  float e0x, e0y, e0z, e1x, e1y, e1z;
  float k0x, k0y, j0x, j0z, k1x, k1y, j1x, j1z;
  PlaneIn<NP, TR, IDPH> in0, in1;
  loadE(ib, e0x, e0y, e0z);
  loadE(ib + 1, e1x, e1y, e1z);
  loadEdge(ib, k0x, k0y, j0x, j0z);
  loadIn(ib, in0);
  float hyp = 0.f, hzp = 0.f;
  if (p.smem) __syncthreads();   // the tables

#pragma unroll 1
  for (int i = ib; i < i1; ++i) {
    // next plane's inputs: E(i + 2), the edges of E(i + 1), H etc. of plane i + 1
    float e2x, e2y, e2z;
    loadE(i + 2, e2x, e2y, e2z);
    loadEdge(i + 1, k1x, k1y, j1x, j1z);
    loadIn(i + 1, in1);
    const bool halo = i < i0;           // H only, for the E update of plane i0
    const bool edo = !halo && i < nx;   // E is formed on this plane

    // ---- H of plane i (h_site's neighbours and ranges)
    xE[w][lane] = make_float2(e0x, e0z);
    __syncthreads();
    const float2 up = top ? make_float2(j0x, j0z) : xE[w + (top ? 0 : 1)][lane];
    float exk = __shfl_down_sync(FULL, e0x, 1);
    float eyk = __shfl_down_sync(FULL, e0y, 1);
    if (lane == 31) {
      exk = k0x;
      eyk = k0y;
    }
    float hx = in0.hx, hy = in0.hy, hz = in0.hz;
    // x-slab membership of the plane; a warp with no node in any slab takes the node code
    // without PML (the same arithmetic there), so the slab code costs only where it applies
    int whEx = 0, prEx = 0, whHx = 0, prHx = 0;
    if (PK != PML_NONE) {
      whEx = axis_member<true>(i, nx, p.slab[0].T, p.slab[3].T, prEx);
      whHx = axis_member<false>(i, nx, p.slab[0].T, p.slab[3].T, prHx);
    }
    {
      const bool iin = i < nx, jin = j < ny, kin = k < nz;
      const float ex_j = jin ? up.x : 0.f;
      const float ez_j = jin ? up.y : 0.f;
      const float ex_k = kin ? exk : 0.f;
      const float ey_k = kin ? eyk : 0.f;
      const float ey_n = iin ? e1y : 0.f;
      const float ez_n = iin ? e1z : 0.f;
      int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
      if (PK != PML_NONE && nodev && iin && jin && kin) {
        where[0] = whHx; pr[0] = prHx;
        where[1] = whHy; pr[1] = prHy;
        where[2] = whHz; pr[2] = prHz;
      }
      const uint32_t wd = in0.ph;
      const bool slab = (where[0] | where[1] | where[2]) != 0;
      if (__any_sync(FULL, slab)) {
        if (nodev)
          h_node<PK, IDPH, false>(p, hc, i, j, k, (smask & 2u) != 0, it, where, pr, ez_j - e0z,
                                  ey_k - e0y, ex_k - e0x, ez_n - e0z, ey_n - e0y, ex_j - e0x,
                                  wd & kPackMask, (wd >> kPackBits) & kPackMask,
                                  (wd >> (2 * kPackBits)) & kPackMask, hx, hy, hz,
                                  own && !halo);
      } else if (nodev) {
        h_node<PML_NONE, IDPH, false>(p, hc, i, j, k, (smask & 2u) != 0, it, where, pr,
                                      ez_j - e0z, ey_k - e0y, ex_k - e0x, ez_n - e0z,
                                      ey_n - e0y, ex_j - e0x, wd & kPackMask,
                                      (wd >> kPackBits) & kPackMask,
                                      (wd >> (2 * kPackBits)) & kPackMask, hx, hy, hz);
      }
    }

    // ---- E of plane i (e_site's neighbours)
    xH[w][lane] = make_float2(hx, hz);
    __syncthreads();
    const float2 dn = xH[w > 0 ? w - 1 : 0][lane];
    const float hxk = __shfl_up_sync(FULL, hx, 1);
    const float hyk = __shfl_up_sync(FULL, hy, 1);
    const bool eslab = edo && eown && PK != PML_NONE && (whEx | whEy | whEz) != 0;
    const bool eslabs = __any_sync(FULL, eslab);
    if (edo && eown) {
      const float hx_j = j >= 1 ? dn.x : 0.f;
      const float hz_j = j >= 1 ? dn.y : 0.f;
      const float hx_k = k >= 1 ? hxk : 0.f;
      const float hy_k = k >= 1 ? hyk : 0.f;
      const float hy_p = i >= 1 ? hyp : 0.f;
      const float hz_p = i >= 1 ? hzp : 0.f;
      const uint32_t wd = in0.pe;
      uint32_t m[3];
      m[0] = wd & kPackMask;
      m[1] = (wd >> kPackBits) & kPackMask;
      m[2] = (wd >> (2 * kPackBits)) & kPackMask;
      float e[3] = {e0x, e0y, e0z};
      int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
      if (PK != PML_NONE) {
        where[0] = whEx; pr[0] = prEx;
        where[1] = whEy; pr[1] = prEy;
        where[2] = whEz; pr[2] = prEz;
      }
      if (eslabs)
        e_node<PK, NP, false, TR>(p, C4, Cs, CD, i, j, k, (smask & 1u) != 0, it, where, pr,
                                  hz - hz_j, hy - hy_k, hx - hx_k, hz - hz_p, hy - hy_p,
                                  hx - hx_j, m, e, in0.t);
      else
        e_node<PML_NONE, NP, false, TR>(p, C4, Cs, CD, i, j, k, (smask & 1u) != 0, it, where,
                                        pr, hz - hz_j, hy - hy_k, hx - hx_k, hz - hz_p,
                                        hy - hy_p, hx - hx_j, m, e, in0.t);
      const int idx = i * sx + col;
      p.En[0][idx] = e[0];
      p.En[1][idx] = e[1];
      p.En[2][idx] = e[2];
      if (NP > 0 && (wd & kDispersiveBit)) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int qq = 0; qq < NP; ++qq) {
            const long long o = (c * NP + qq) * (long long)p.ncomp + idx;
            if (TR) reinterpret_cast<float*>(p.T)[o] = in0.t[c][qq].x;
            else p.T[o] = in0.t[c][qq];
          }
      }
    }
    if (!halo && own) {
      const int idx = i * sx + col;
      p.Hn[0][idx] = hx;
      p.Hn[1][idx] = hy;
      p.Hn[2][idx] = hz;
    }
    // the next plane
    hyp = hy;
    hzp = hz;
    e0x = e1x; e0y = e1y; e0z = e1z;
    e1x = e2x; e1y = e2y; e1z = e2z;
    k0x = k1x; k0y = k1y; j0x = j1x; j0z = j1z;
    in0 = in1;
  }
}

}  // namespace gbf
