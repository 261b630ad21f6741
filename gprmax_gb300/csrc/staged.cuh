// staged.cuh — the H and E half-steps with their inputs staged in shared memory by bulk copies.
//
// The plain half-steps (h_half_step, e_half_step, fdtd_kernels.cuh) load every input of a node
// in the thread that updates it; with the registers the node code needs, the loads a warp has
// in flight do not cover the memory latency and the kernels wait on them. Here one thread of
// each block copies whole chunks of consecutive nodes — for E: E, H and H's k-1, j-1 and i-1
// neighbours, the packed material word and the pole state; for H: H, E and E's k+1, j+1 and
// i+1 neighbours and the packed word; and the z slabs' Phi state of the chunk's rows — into a
// ring of shared-memory stages with cp.async.bulk,
// each chunk's copies completing one mbarrier phase, several chunks ahead of the warps that
// update them; those read their operands from shared memory (the PML profile rows too, copied
// once per block; the x and y slabs' Phi state, on few chunks, is read where it lies). The
// block is one producer warp
// and kStagedC consumer warps: a consumer warp waits for a stage's "full" barrier, updates its
// nodes and arrives on the stage's "empty" barrier; the producer refills a stage once every
// consumer warp has arrived. No barrier spans the block, so a warp held up by slab nodes delays
// no other until the ring runs dry. The node arithmetic is h_node's and e_node's
// (update_magnetic, update_electric / update_electric_dispersive_*, the PML corrections,
// sources, part B: fields_updates_ext.pyx:30-412), so the results are the plain kernels' bit for
// bit.
//
// Chunks: the domain is taken plane by plane — for E (i < nx, j < ny, k < nz) plane i is the
// run of nodes [i*sx, i*sx + ny*sy) (the k = nz node that ends each row is skipped), for H
// (every node) the whole plane [i*sx, (i+1)*sx) — cut into chunks of kStageL nodes that start
// on 4-node boundaries. Chunk c covers plane c / cpp; blocks take chunks c = blockIdx.x,
// blockIdx.x + gridDim.x, ..., so the whole grid streams the arrays front to back. A chunk
// whose nodes all lie in the core ranges along x and y (the plain kernels' core box) runs the
// core node code (only the z slabs to test); the others run the general code.
//
// Every copy moves kStageSpan floats (twice that, from twice the offset, for a complex pole
// state's (re, im) pairs) from a 16-byte-aligned start: the device arrays start on 256-byte
// boundaries (their stride is a multiple of 64 nodes) and every start is a multiple of 4
// nodes, clamped into [0, amax] so that a copy never leaves its array; a node reads a neighbour
// only where the plain kernel does, and such values always lie inside the copied span. Waits
// are bounded: a stage not filled within the limit sets the error word, the block waits (again
// bounded) for its copies in flight and returns; launches that find the word set return at once.
#pragma once
#include "fdtd_kernels.cuh"

namespace gbf {

// Launch shape: a producer warp and kStagedC consumer warps (1024 threads, one block per SM),
// one node per consumer thread per chunk: chunks of kStageL nodes, copies of kStageSpan floats.
// Measured on the GB300 (400 x 400 x 200 Debye soil, E half-step): 16 consumer warps with two
// nodes each 0.53 ms, 24 warps 0.47 ms, 31 warps 0.41 ms; the plain kernel 0.45 ms.
constexpr int kStagedC = 31;
constexpr int kStagedThreads = 32 * (kStagedC + 1);
constexpr int kStageL = 32 * kStagedC;
constexpr int kStageSpan = kStageL + 8;
constexpr int kStageMax = 4;   // deepest ring
// streams of an E chunk, each kStageSpan floats in a stage: E own (3), H own from node s - 4
// (3), Hx, Hz at s - sy (2), Hy, Hz at s - sx (2), the packed E word (1), the pole state (3 NP
// with its real parts only; 6 NP for complex state: each component and pole's (re, im) pairs
// take two stream slots)
constexpr int kStE = 0, kStH = 3, kStJ = 6, kStI = 8, kStPE = 10, kStT = 11;
// streams of an H chunk: E own (3), H own (3), Ex, Ez at s + sy (2), Ey, Ez at s + sx (2), the
// packed H word (1, when the H half-step reads IDs)
constexpr int kHtE = 0, kHtH = 3, kHtJ = 6, kHtI = 8, kHtP = 10;

// Division of a non-negative int n < 2^31 by a constant d >= 2 as a multiply-high and a shift
// (Granlund and Montgomery, "Division by invariant integers using multiplication", PLDI 1994,
// theorem 4.2 with N = 31): with l = ceil(log2 d) and m = ceil(2^(31+l) / d) < 2^32,
// n / d = (n * m) >> (31 + l).
struct FastDiv {
  uint32_t m;
  int sh;   // l - 1: the shift after the high word of the product
  __device__ __forceinline__ int div(int n) const {
    return (int)(__umulhi((uint32_t)n, m) >> sh);
  }
};

struct StagedGeom {
  int cpp;              // chunks per plane
  int nchunks;          // planes * cpp (nx planes for E, nx + 1 for H)
  int nstages;          // stages in the ring (2 .. kStageMax)
  int nstream;          // streams per chunk: E 11 + 3 NP (6 NP complex), H 10 (11 with packed H IDs)
  int ilo, ihi;         // core range along x (the plain kernel's core box)
  int jlo, jhi;         // and along y
  int amax;             // largest copy start (nodes) keeping a copy inside its array
  int ring_off;         // byte offset of the ring in dynamic shared memory (after the rows)
  int stage_floats;     // floats per stage: nstream * kStageSpan + zslots * zspan
  int zslots;           // z-slab Phi copies per chunk: 2 sides x 2 arrays x CFS order (or 0)
  int zspan;            // floats per z-slab Phi copy
  int rows_off;         // byte offset of the PML profile rows in dynamic shared memory
  int roff[6];          // float offset of each slab's rows there ([4][order][T], the kernel's
                        // field type: eR for E, hR for H)
  FastDiv by_sy;        // n / sy
  FastDiv by_cpp;       // n / cpp (cpp >= 2; unused when cpp == 1)
  int* err;             // set to 1 when a wait for a stage runs out
  long long limit_ns;   // wait limit
};

typedef void (*SKernFn)(StepParams, StagedGeom);
// per-kind tables (staged_inst.cu): the staged E kernel for `np` poles (real state) and the
// staged H kernel for ID layout `idp` (0: one H row for every material, 1: packed), or NULL
void staged_pk0(int np, int treal, int idp, SKernFn* e, SKernFn* h);
void staged_pk1(int np, int treal, int idp, SKernFn* e, SKernFn* h);
void staged_pk2(int np, int treal, int idp, SKernFn* e, SKernFn* h);
void staged_pk3(int np, int treal, int idp, SKernFn* e, SKernFn* h);
void staged_pk4(int np, int treal, int idp, SKernFn* e, SKernFn* h);

__device__ __forceinline__ uint32_t smem_addr(const void* q) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(q));
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void proxy_async_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}
// one arrival that also expects `bytes` of copies to complete the phase
__device__ __forceinline__ void mbar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes) : "memory");
}
// global -> shared bulk copy completing on barrier b (both addresses 16-byte aligned, bytes a
// multiple of 16)
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done) : "r"(smem_addr(b)), "r"(parity) : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase with parity `parity` of barrier b to complete, at most limit_ns; gives up
// early once *abort is set.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, long long limit_ns,
                                          const volatile int* abort) {
  if (mbar_test(b, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_test(b, parity))
    if (*abort || (long long)(global_ns() - t0) > limit_ns) return false;
  return true;
}

// Where chunk c lies, as the producer writes it into the stage's header for the consumers:
// plane i, first node s (a multiple of 4), where node s of each stream group lies in its stream
// (shE for the own E and H of an H chunk, E, the packed word and the pole state of an E chunk;
// shH own H of an E chunk; shJ the j neighbours, shI the i neighbours), row jf and column kf of
// node s in the plane (jf = -1 for the up to three nodes before the plane's first), and whether
// every node of the chunk lies in the core box; zst: the first Phi element of each z-slab copy
// (z minus, z plus) x (CFS order 1, 2), as an index into the slab's Phi arrays.
// (rows of 16 ints on 16-byte boundaries, so that a consumer reads its header in four vector
// loads)
enum { kHdrI, kHdrS, kHdrShE, kHdrShH, kHdrShJ, kHdrShI, kHdrJ, kHdrK, kHdrCore, kHdrZ,
       kHdrInts = 16 };
static_assert(kHdrZ + 4 <= kHdrInts, "header row");

__device__ __forceinline__ int clamp_start(int a, int amax) {
  return a < 0 ? 0 : (a > amax ? amax : a);
}

// The producer: copy chunk c into stage `st` of the ring and describe it in the header h.
// E chunks take their H neighbours at s - 1, s - sy, s - sx; H chunks their E neighbours at
// s + 1, s + sy, s + sx.
template <bool ELECTRIC, int PK, int NP, bool TR, int IDP>
__device__ __forceinline__ void stage_chunk(const StepParams& p, const StagedGeom& g, float* ring,
                                            uint64_t* bar, int* h, int c, int st) {
  constexpr int W = kStageSpan;
  const int i = g.cpp == 1 ? c : g.by_cpp.div(c);
  const int s = ((i * p.sx) & ~3) + (c - i * g.cpp) * kStageL;
  const int dj = ELECTRIC ? -p.sy : p.sy, di = ELECTRIC ? -p.sx : p.sx;
  const int aE = clamp_start(s, g.amax);
  const int aH = clamp_start(ELECTRIC ? s - 4 : s, g.amax);
  const int aJ = clamp_start((s + dj) & ~3, g.amax);   // & ~3 rounds down, negatives included
  const int aI = clamp_start((s + di) & ~3, g.amax);
  const int f = s - i * p.sx;
  const int jf = f >= 0 ? g.by_sy.div(f) : -1;
  const int plen = ELECTRIC ? p.ny * p.sy : p.sx;
  const int jl = g.by_sy.div(f + kStageL - 1 < plen ? f + kStageL - 1 : plen - 1);
  h[kHdrI] = i;
  h[kHdrS] = s;
  h[kHdrShE] = s - aE;
  h[kHdrShH] = s - aH;
  h[kHdrShJ] = s + dj - aJ;
  h[kHdrShI] = s + di - aI;
  h[kHdrJ] = jf;
  h[kHdrK] = f - jf * p.sy;
  h[kHdrCore] = i >= g.ilo && i < g.ihi && jf >= g.jlo && jl < g.jhi;
  // the z slabs' Phi state of the chunk's rows (Phi index (i * ny + j) * T + pr): one short
  // range per slab, array and CFS order; H nodes on plane nx have no PML update
  constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  const int j0 = jf > 0 ? jf : 0, j1 = jl < p.ny - 1 ? jl : p.ny - 1;
  const bool zrows = g.zslots && j0 <= j1 && (ELECTRIC || i < p.nx);
  int zcopies = 0;
  if (zrows)
    for (int side = 0; side < 2; ++side) zcopies += p.slab[2 + 3 * side].T ? 2 * order : 0;
  // the z copies' first elements, written to the header before the arrival below releases it
  if (zrows) {
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const Slab& sl = p.slab[2 + 3 * side];
#pragma unroll
      for (int o = 0; o < order; ++o)
        h[kHdrZ + 2 * side + o] = ((i * p.ny + j0) * sl.T + o * sl.ocount) & ~3;
    }
  }
  constexpr uint32_t bytes = W * sizeof(float);
  float* d = ring + (size_t)st * g.stage_floats;
  // the arrival releases the header to the consumers that wait on this phase
  mbar_expect(bar, bytes * (uint32_t)g.nstream + (uint32_t)(zcopies * g.zspan) * 4u);
  if (zrows) {
    float* z = d + g.nstream * W;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const Slab& sl = p.slab[2 + 3 * side];
      if (!sl.T) continue;
#pragma unroll
      for (int o = 0; o < order; ++o) {
        const int a = h[kHdrZ + 2 * side + o];
        const float* src1 = ELECTRIC ? sl.phiE1 : sl.phiH1;
        const float* src2 = ELECTRIC ? sl.phiE2 : sl.phiH2;
        bulk_copy(z + ((side * 2 + 0) * order + o) * g.zspan, src1 + a, g.zspan * 4u, bar);
        bulk_copy(z + ((side * 2 + 1) * order + o) * g.zspan, src2 + a, g.zspan * 4u, bar);
      }
    }
  }
  if (ELECTRIC) {
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      bulk_copy(d + (kStE + comp) * W, p.E[comp] + aE, bytes, bar);
      bulk_copy(d + (kStH + comp) * W, p.H[comp] + aH, bytes, bar);
    }
    bulk_copy(d + (kStJ + 0) * W, p.H[0] + aJ, bytes, bar);
    bulk_copy(d + (kStJ + 1) * W, p.H[2] + aJ, bytes, bar);
    bulk_copy(d + (kStI + 0) * W, p.H[1] + aI, bytes, bar);
    bulk_copy(d + (kStI + 1) * W, p.H[2] + aI, bytes, bar);
    bulk_copy(d + kStPE * W, p.PE + aE, bytes, bar);
    const float* T = reinterpret_cast<const float*>(p.T);
#pragma unroll
    if (TR) {
      for (int qq = 0; qq < 3 * NP; ++qq)
        bulk_copy(d + (kStT + qq) * W, T + (long long)qq * p.ncomp + aE, bytes, bar);
    } else {
      // complex state: (re, im) pairs, twice the floats from twice the offset
#pragma unroll
      for (int qq = 0; qq < 3 * NP; ++qq)
        bulk_copy(d + (kStT + 2 * qq) * W, T + 2 * ((long long)qq * p.ncomp + aE), 2 * bytes, bar);
    }
  } else {
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      bulk_copy(d + (kHtE + comp) * W, p.E[comp] + aE, bytes, bar);
      bulk_copy(d + (kHtH + comp) * W, p.H[comp] + aH, bytes, bar);
    }
    bulk_copy(d + (kHtJ + 0) * W, p.E[0] + aJ, bytes, bar);
    bulk_copy(d + (kHtJ + 1) * W, p.E[2] + aJ, bytes, bar);
    bulk_copy(d + (kHtI + 0) * W, p.E[1] + aI, bytes, bar);
    bulk_copy(d + (kHtI + 1) * W, p.E[2] + aI, bytes, bar);
    if (IDP == 1) bulk_copy(d + kHtP * W, p.PH + aE, bytes, bar);
  }
}

// A slab's profile row at index pr from the rows staged in shared memory (load_row's layout).
template <int PK>
__device__ __forceinline__ PmlRow load_row_s(const float* R, int T, int pr) {
  constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  PmlRow c;
  c.RA0 = R[(0 * order + 0) * T + pr];
  c.RB0 = R[(1 * order + 0) * T + pr];
  c.RE0 = R[(2 * order + 0) * T + pr];
  c.RF0 = R[(3 * order + 0) * T + pr];
  if (order == 2) {
    c.RA1 = R[(0 * order + 1) * T + pr];
    c.RB1 = R[(1 * order + 1) * T + pr];
    c.RE1 = R[(2 * order + 1) * T + pr];
    c.RF1 = R[(3 * order + 1) * T + pr];
  } else {
    c.RA1 = c.RB1 = c.RE1 = c.RF1 = 0.f;
  }
  return c;
}

// pml_axis with the profile rows from shared memory and, for the z axis, the Phi state from the
// chunk's stage (z: that stage's z-slab area, hz: its header's copy starts); the x and y Phi
// state is read from global memory. The next state is written to global memory. Same
// arithmetic as pml_axis.
template <int PK, bool ELECTRIC, int AX>
__device__ __forceinline__ void pml_axis_st(const StepParams& p, const StagedGeom& g,
                                            const float* rows, const float* z, const int* hz,
                                            int where, int pr, int i, int j, int k, float dA,
                                            float dB, float& XA, float& XB) {
  constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  const Slab& m = p.slab[AX];
  const Slab& q = p.slab[AX + 3];
  const bool plus = where == 2;
  const int T = plus ? q.T : m.T;
  const int pidx = phi_index<AX>(i, j, k, pr, T, p.ny, p.nz);
  const PmlRow c = load_row_s<PK>(rows + (plus ? g.roff[AX + 3] : g.roff[AX]), T, pr);
  const float d = m.d, r = m.rcp;
  const int fast = m.fastdiv;
  const int ocount = plus ? q.ocount : m.ocount;
  float* out1 = ELECTRIC ? (plus ? q.phiE1 : m.phiE1) : (plus ? q.phiH1n : m.phiH1n);
  float* out2 = ELECTRIC ? (plus ? q.phiE2 : m.phiE2) : (plus ? q.phiH2n : m.phiH2n);
  float a0, a1 = 0.f, b0, b1 = 0.f;
  if (AX == 2) {
    const int side = plus ? 1 : 0;
    const float* zs = z + side * 2 * order * g.zspan;
    a0 = zs[pidx - hz[2 * side]];
    b0 = zs[order * g.zspan + pidx - hz[2 * side]];
    if (order == 2) {
      a1 = zs[g.zspan + pidx + ocount - hz[2 * side + 1]];
      b1 = zs[3 * g.zspan + pidx + ocount - hz[2 * side + 1]];
    }
  } else {
    const float* in1 = ELECTRIC ? out1 : (plus ? q.phiH1 : m.phiH1);
    const float* in2 = ELECTRIC ? out2 : (plus ? q.phiH2 : m.phiH2);
    a0 = in1[pidx];
    b0 = in2[pidx];
    if (order == 2) {
      a1 = in1[pidx + ocount];
      b1 = in2[pidx + ocount];
    }
  }
  XA = pml_update_v<PK>(div_cell(dA, d, r, fast), a0, a1, out1, pidx, ocount, c, true);
  XB = pml_update_v<PK>(div_cell(dB, d, r, fast), b0, b1, out2, pidx, ocount, c, true);
}

// One H node from a stage: the operands h_site loads from global memory, read from shared memory.
template <int PK, int IDP, bool CORE>
__device__ __forceinline__ void h_site_staged(const StepParams& p, const StagedGeom& g,
                                              const HCoef& hc, const float* rows,
                                              const float* __restrict__ S, const int* h, int shE,
                                              int shJ, int shI, int r, int i, int j, int k,
                                              int idx, int it) {
  static_assert(IDP == 0 || IDP == 1, "the staged H sweep reads packed IDs or none");
  constexpr int W = kStageSpan;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const float* sE = S + kHtE * W + shE + r;   // E, H and the packed word share the same start
  const float* sJ = S + kHtJ * W + shJ + r;
  const float* sI = S + kHtI * W + shI + r;
  const bool iin = CORE || i < nx, jin = CORE || j < ny, kin = k < nz;
  const float ex_c = sE[0], ey_c = sE[W], ez_c = sE[2 * W];
  const float ex_j = jin ? sJ[0] : 0.f;
  const float ez_j = jin ? sJ[W] : 0.f;
  const float ex_k = kin ? sE[1] : 0.f;
  const float ey_k = kin ? sE[W + 1] : 0.f;
  const float ey_n = iin ? sI[0] : 0.f;
  const float ez_n = iin ? sI[W] : 0.f;
  uint32_t mx = 0, my = 0, mz = 0;
  if (IDP == 1) {
    const uint32_t w = __float_as_uint(sE[(kHtP - kHtE) * W]);
    mx = w & kPackMask;
    my = (w >> kPackBits) & kPackMask;
    mz = (w >> (2 * kPackBits)) & kPackMask;
  }
  float hx = sE[(kHtH - kHtE) * W], hy = sE[(kHtH - kHtE + 1) * W], hz = sE[(kHtH - kHtE + 2) * W];
  int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
  if (PK != PML_NONE && iin && jin && kin) {
    if (!CORE) {
      where[0] = axis_member<false>(i, nx, p.slab[0].T, p.slab[3].T, pr[0]);
      where[1] = axis_member<false>(j, ny, p.slab[1].T, p.slab[4].T, pr[1]);
    }
    where[2] = axis_member<false>(k, nz, p.slab[2].T, p.slab[5].T, pr[2]);
  }
  const bool src = p.nsrcH && node_has_source(idx, p.nsrcH, p.srcqH, p.srcH, p.sx, p.sy);
  const float dEz_y = ez_j - ez_c, dEy_z = ey_k - ey_c, dEx_z = ex_k - ex_c;
  const float dEz_x = ez_n - ez_c, dEy_x = ey_n - ey_c, dEx_y = ex_j - ex_c;
  float XA[3] = {0.f, 0.f, 0.f}, XB[3] = {0.f, 0.f, 0.f};
  if (PK != PML_NONE) {
    const float* z = S + g.nstream * kStageSpan;
    if (!CORE && where[0]) pml_axis_st<PK, false, 0>(p, g, rows, z, h + kHdrZ, where[0], pr[0], i, j, k, dEz_x, dEy_x, XA[0], XB[0]);
    if (!CORE && where[1]) pml_axis_st<PK, false, 1>(p, g, rows, z, h + kHdrZ, where[1], pr[1], i, j, k, dEz_y, dEx_y, XA[1], XB[1]);
    if (where[2]) pml_axis_st<PK, false, 2>(p, g, rows, z, h + kHdrZ, where[2], pr[2], i, j, k, dEy_z, dEx_z, XA[2], XB[2]);
  }
  h_node_x<PK, IDP, CORE, true>(p, hc, i, j, k, src, it, where, XA, XB, dEz_y, dEy_z, dEx_z, dEz_x,
                          dEy_x, dEx_y, mx, my, mz, hx, hy, hz);
  p.H[0][idx] = hx;
  p.H[1][idx] = hy;
  p.H[2][idx] = hz;
}

// One E node from a stage: the operands e_site loads from global memory, read from shared memory
// (S: the stage; shE, shH, shJ, shI: where node s of each stream group lies in its stream).
template <int PK, int NP, bool CORE, bool TR>
__device__ __forceinline__ void e_site_staged(const StepParams& p, const StagedGeom& g,
                                              const float4* C4, const float* Cs, const float2* CD,
                                              const float* rows, const float* __restrict__ S,
                                              const int* h, int shE, int shH, int shJ, int shI,
                                              int r, int i, int j, int k, int idx, int it) {
  constexpr int NPV = NP > 0 ? NP : 1;
  constexpr int W = kStageSpan;
  const float* sE = S + kStE * W + shE + r;   // E, the packed word and T share the E start
  const float* sH = S + kStH * W + shH + r;
  const float* sJ = S + kStJ * W + shJ + r;
  const float* sI = S + kStI * W + shI + r;
  const float hx_c = sH[0], hy_c = sH[W], hz_c = sH[2 * W];
  const float hx_j = (CORE || j >= 1) ? sJ[0] : 0.f;
  const float hz_j = (CORE || j >= 1) ? sJ[W] : 0.f;
  const float hx_k = k >= 1 ? sH[-1] : 0.f;
  const float hy_k = k >= 1 ? sH[W - 1] : 0.f;
  const float hy_p = (CORE || i >= 1) ? sI[0] : 0.f;
  const float hz_p = (CORE || i >= 1) ? sI[W] : 0.f;
  const uint32_t w = __float_as_uint(sE[(kStPE - kStE) * W]);
  uint32_t m[3];
  m[0] = w & kPackMask;
  m[1] = (w >> kPackBits) & kPackMask;
  m[2] = (w >> (2 * kPackBits)) & kPackMask;
  const bool disp = NP > 0 && (w & kDispersiveBit);
  float e[3];
  float2 t[3][NPV];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    e[comp] = sE[comp * W];
#pragma unroll
    for (int qq = 0; qq < NP; ++qq)
      t[comp][qq] = TR ? make_float2(sE[(kStT - kStE + comp * NP + qq) * W], 0.f)
                       : *reinterpret_cast<const float2*>(S + (kStT + 2 * (comp * NP + qq)) * W +
                                                          2 * (shE + r));
  }
  int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
  if (PK != PML_NONE) {
    if (!CORE) {
      where[0] = axis_member<true>(i, p.nx, p.slab[0].T, p.slab[3].T, pr[0]);
      where[1] = axis_member<true>(j, p.ny, p.slab[1].T, p.slab[4].T, pr[1]);
    }
    where[2] = axis_member<true>(k, p.nz, p.slab[2].T, p.slab[5].T, pr[2]);
  }
  const bool src = p.nsrcE && node_has_source(idx, p.nsrcE, p.srcqE, p.srcE, p.sx, p.sy);
  const float dHz_y = hz_c - hz_j, dHy_z = hy_c - hy_k, dHx_z = hx_c - hx_k;
  const float dHz_x = hz_c - hz_p, dHy_x = hy_c - hy_p, dHx_y = hx_c - hx_j;
  float XA[3] = {0.f, 0.f, 0.f}, XB[3] = {0.f, 0.f, 0.f};
  if (PK != PML_NONE) {
    const float* z = S + g.nstream * kStageSpan;
    if (!CORE && where[0]) pml_axis_st<PK, true, 0>(p, g, rows, z, h + kHdrZ, where[0], pr[0], i, j, k, dHz_x, dHy_x, XA[0], XB[0]);
    if (!CORE && where[1]) pml_axis_st<PK, true, 1>(p, g, rows, z, h + kHdrZ, where[1], pr[1], i, j, k, dHz_y, dHx_y, XA[1], XB[1]);
    if (where[2]) pml_axis_st<PK, true, 2>(p, g, rows, z, h + kHdrZ, where[2], pr[2], i, j, k, dHy_z, dHx_z, XA[2], XB[2]);
  }
  e_node_x<PK, NP, CORE, TR>(p, C4, Cs, CD, i, j, k, src, it, where, XA, XB, m, e, t, dHz_y, dHy_z,
                             dHx_z, dHz_x, dHy_x, dHx_y);
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    p.E[comp][idx] = e[comp];
    if (disp) {
#pragma unroll
      for (int qq = 0; qq < NP; ++qq) {
        const long long o = (comp * NP + qq) * (long long)p.ncomp + idx;
        if (TR) reinterpret_cast<float*>(p.T)[o] = t[comp][qq].x;
        else p.T[o] = t[comp][qq];
      }
    }
  }
}

// The producer/consumer sweep of one half-step (ELECTRIC: E, else H) over its chunks.
template <bool ELECTRIC, int PK, int NP, bool TR, int IDP>
__device__ __forceinline__ void staged_sweep(const StepParams& p, const StagedGeom& g) {
  extern __shared__ __align__(128) float4 smem_st[];
  __shared__ uint64_t full[kStageMax], empty[kStageMax];
  __shared__ __align__(16) int hdr[kStageMax][kHdrInts];
  __shared__ int abort_flag;
  // after a sweep that gave up, the run's fields are void: later launches return at once, until
  // the host has read and cleared the error word
  if (*static_cast<volatile int*>(g.err)) return;
  float4* s4;
  float* ss;
  float2* sd = nullptr;
  if (ELECTRIC) {
    e_tables(p, smem_st, s4, ss, sd);
  } else {
    s4 = smem_st;
    ss = reinterpret_cast<float*>(s4 + (p.smem ? p.nmat : 0));
  }
  float* ring = reinterpret_cast<float*>(reinterpret_cast<char*>(smem_st) + g.ring_off);
  float* rows = reinterpret_cast<float*>(reinterpret_cast<char*>(smem_st) + g.rows_off);
  const int G = gridDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* abortp = &abort_flag;
  if (threadIdx.x == 0) {
    for (int q = 0; q < g.nstages; ++q) {
      mbar_init(&full[q], 1);
      mbar_init(&empty[q], kStagedC);
    }
    abort_flag = 0;
    mbar_init_fence();
  }
  if (p.smem) stage_tables(p, ELECTRIC, s4, ss, ELECTRIC && NP > 0 ? sd : nullptr);
  if (PK != PML_NONE) {
    constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
    for (int sl = 0; sl < 6; ++sl) {
      const Slab& b = p.slab[sl];
      const float* src = ELECTRIC ? b.eR : b.hR;
      for (int q = threadIdx.x; q < 4 * order * b.T; q += blockDim.x) rows[g.roff[sl] + q] = __ldg(src + q);
    }
  }
  __syncthreads();
  if (warp == 0) {
    // the producer: lane 0 fills the ring, a stage again once all consumer warps left it
    if (lane != 0) return;
    // chunk n goes to stage st = n % nstages in round n / nstages; from the second round on it
    // waits for the phase of the round before (parity of round - 1), counted as it goes
    int n = 0, st = 0;
    uint32_t round = 0;
    for (int c = blockIdx.x; c < g.nchunks; c += G, ++n) {
      if (round > 0 && !mbar_wait(&empty[st], (round - 1) & 1u, g.limit_ns, abortp)) {
        *abortp = 1;
        atomicOr(g.err, 1);
        break;
      }
      // the consumers' reads of this stage are ordered before the copies that refill it
      proxy_async_fence();
      stage_chunk<ELECTRIC, PK, NP, TR, IDP>(p, g, ring, &full[st], hdr[st], c, st);
      if (++st == g.nstages) {
        st = 0;
        ++round;
      }
    }
    // on giving up: let the copies in flight (the latest chunk of each stage) land before the
    // block may end
    if (*abortp) {
      const volatile int keep_waiting = 0;
      for (int m = n - 1; m >= 0 && m >= n - g.nstages; --m)
        mbar_wait(&full[m % g.nstages], (uint32_t)(m / g.nstages) & 1u, g.limit_ns, &keep_waiting);
    }
    return;
  }
  // a consumer thread updates node t of every chunk: its row and column offsets from the
  // chunk's first node
  const int t = threadIdx.x - 32;
  const int tq = g.by_sy.div(t), tr = t - tq * p.sy;
  const int it = ELECTRIC ? (p.nsrcE ? *p.d_it : 0) : (p.nsrcH ? *p.d_it : 0);
  const int jend = ELECTRIC ? p.ny : p.ny + 1, kend = ELECTRIC ? p.nz : p.sy;
  HCoef hc;
  hc.C4 = p.smem ? s4 : p.cH4;
  hc.Cs = p.smem ? ss : p.cHs;
  const float4* C4 = p.smem ? s4 : p.cE4;
  const float* Cs = p.smem ? ss : p.cEs;
  const float2* CD = (p.smem && NP > 0) ? sd : p.cD;
  // stage and phase parity of the next chunk, counted as it goes (no division per chunk)
  int st = 0;
  uint32_t parity = 0;
  const float* S = ring;   // stage st
  for (int c = blockIdx.x; c < g.nchunks; c += G) {
    if (!mbar_wait(&full[st], parity, g.limit_ns, abortp)) {
      *abortp = 1;
      atomicOr(g.err, 1);
      return;
    }
    const int* h = hdr[st];
    // the header's first twelve entries in three vector loads
    const int4 ha = reinterpret_cast<const int4*>(h)[0];   // i, s, shE, shH
    const int4 hb = reinterpret_cast<const int4*>(h)[1];   // shJ, shI, jf, kf
    const int4 hc4 = reinterpret_cast<const int4*>(h)[2];  // core, z starts
    static_assert(kHdrI == 0 && kHdrS == 1 && kHdrShE == 2 && kHdrShH == 3 && kHdrShJ == 4 &&
                  kHdrShI == 5 && kHdrJ == 6 && kHdrK == 7 && kHdrCore == 8, "header layout");
    const int i = ha.x, s = ha.y;
    int j = hb.z + tq, k = hb.w + tr;
    if (k >= p.sy) { k -= p.sy; ++j; }
    if (j >= 0 && j < jend && k < kend) {
      if (ELECTRIC) {
        if (hc4.x)
          e_site_staged<PK, NP, true, TR>(p, g, C4, Cs, CD, rows, S, h, ha.z, ha.w, hb.x, hb.y,
                                          t, i, j, k, s + t, it);
        else
          e_site_staged<PK, NP, false, TR>(p, g, C4, Cs, CD, rows, S, h, ha.z, ha.w, hb.x, hb.y,
                                           t, i, j, k, s + t, it);
      } else {
        if (hc4.x)
          h_site_staged<PK, IDP, true>(p, g, hc, rows, S, h, ha.z, hb.x, hb.y, t, i, j, k, s + t,
                                       it);
        else
          h_site_staged<PK, IDP, false>(p, g, hc, rows, S, h, ha.z, hb.x, hb.y, t, i, j, k,
                                        s + t, it);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
    S += g.stage_floats;
    if (++st == g.nstages) {
      st = 0;
      parity ^= 1u;
      S = ring;
    }
  }
}

template <int PK, int NP, bool TR>
__global__ void __launch_bounds__(kStagedThreads, 1)
e_half_step_staged(const __grid_constant__ StepParams p, const __grid_constant__ StagedGeom g) {
  staged_sweep<true, PK, NP, TR, 1>(p, g);
}

template <int PK, int IDP>
__global__ void __launch_bounds__(kStagedThreads, 1)
h_half_step_staged(const __grid_constant__ StepParams p, const __grid_constant__ StagedGeom g) {
  staged_sweep<false, PK, 0, false, IDP>(p, g);
}

}  // namespace gbf
