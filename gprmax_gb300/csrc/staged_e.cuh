// staged_e.cuh — the E half-step with its inputs staged in shared memory by bulk copies.
//
// The plain E half-step (e_half_step, fdtd_kernels.cuh) loads every input of a node in the
// thread that updates it; with the registers the node code needs, the loads a warp has in flight
// do not cover the memory latency and the kernel waits on them. Here one thread of each block
// copies whole chunks of consecutive nodes — E, H and H's k-1, j-1 and i-1 neighbours, the
// packed material word and the pole state — into a ring of shared-memory stages with
// cp.async.bulk, each chunk's copies completing one mbarrier phase, several chunks ahead of the
// warps that update them; those read their operands from shared memory. The block is one
// producer warp and C consumer warps: a consumer warp waits for a stage's "full" barrier,
// updates its nodes and arrives on the stage's "empty" barrier; the producer refills a stage
// once every consumer warp has arrived. No barrier spans the block, so a warp held up by slab
// nodes delays no other until the ring runs dry. The node
// arithmetic is e_node's (update_electric / update_electric_dispersive_*, the PML corrections,
// sources, part B: fields_updates_ext.pyx:30-349), so the results are the plain kernel's bit for
// bit.
//
// Chunks: the E domain (i < nx, j < ny, k < nz) is taken plane by plane, plane i being the run
// of nodes [i*sx, i*sx + ny*sy) (the k = nz node that ends each row is skipped), cut into chunks
// of L nodes that start on 4-node boundaries. Chunk c covers plane c / cpp; blocks take
// chunks c = blockIdx.x, blockIdx.x + gridDim.x, ..., so the whole grid streams the arrays front
// to back. A chunk whose nodes all lie in the core ranges along x and y (the plain kernel's core
// box) runs the core node code (only the z slabs to test); the others run the general code.
//
// Every copy moves L + 8 floats from a 16-byte-aligned start: the device arrays start on
// 256-byte boundaries (their stride is a multiple of 64 nodes) and every start is a multiple of 4
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
// streams of a chunk, each L + 8 floats in a stage: E own (3), H own from node s - 4 (3),
// Hx, Hz at s - sy (2), Hy, Hz at s - sx (2), the packed E word (1), the pole state (3 * NP)
constexpr int kStE = 0, kStH = 3, kStJ = 6, kStI = 8, kStPE = 10, kStT = 11;

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
  int nchunks;          // nx * cpp
  int nstages;          // stages in the ring (2 .. kStageMax)
  int nstream;          // streams per chunk, 11 + 3 * NP
  int ilo, ihi;         // core range along x (the plain kernel's core box)
  int jlo, jhi;         // and along y
  int amax;             // largest copy start (nodes) keeping a copy inside its array
  int ring_off;         // byte offset of the ring in dynamic shared memory (after the tables)
  FastDiv by_sy;        // n / sy
  FastDiv by_cpp;       // n / cpp (cpp >= 2; unused when cpp == 1)
  int* err;             // set to 1 when a wait for a stage runs out
  long long limit_ns;   // wait limit
};

typedef void (*SKernFn)(StepParams, StagedGeom);
// per-kind tables (staged_inst.cu): the staged kernel for `np` poles (real state), or NULL
void staged_pk0(int np, int treal, SKernFn* e);
void staged_pk1(int np, int treal, SKernFn* e);
void staged_pk2(int np, int treal, SKernFn* e);
void staged_pk3(int np, int treal, SKernFn* e);
void staged_pk4(int np, int treal, SKernFn* e);

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
// (shE for E, the packed word and the pole state; shH own H; shJ H at s - sy; shI H at s - sx),
// row jf and column kf of node s in the plane (jf = -1 for the up to three nodes before the
// plane's first), and whether every node of the chunk lies in the core box.
enum { kHdrI, kHdrS, kHdrShE, kHdrShH, kHdrShJ, kHdrShI, kHdrJ, kHdrK, kHdrCore, kHdrInts = 12 };

__device__ __forceinline__ int clamp_start(int a, int amax) {
  return a < 0 ? 0 : (a > amax ? amax : a);
}

// The producer: copy chunk c into stage `st` of the ring and describe it in the header h.
template <int NP>
__device__ __forceinline__ void stage_chunk(const StepParams& p, const StagedGeom& g, float* ring,
                                            uint64_t* bar, int* h, int c, int st) {
  constexpr int W = kStageSpan;
  const int i = g.cpp == 1 ? c : g.by_cpp.div(c);
  const int s = ((i * p.sx) & ~3) + (c - i * g.cpp) * kStageL;
  const int aE = clamp_start(s, g.amax);
  const int aH = clamp_start(s - 4, g.amax);
  const int aJ = clamp_start((s - p.sy) & ~3, g.amax);   // & ~3 rounds down, negatives included
  const int aI = clamp_start((s - p.sx) & ~3, g.amax);
  const int f = s - i * p.sx;
  const int jf = f >= 0 ? g.by_sy.div(f) : -1;
  const int plen = p.ny * p.sy;
  const int jl = g.by_sy.div(f + kStageL - 1 < plen ? f + kStageL - 1 : plen - 1);
  h[kHdrI] = i;
  h[kHdrS] = s;
  h[kHdrShE] = s - aE;
  h[kHdrShH] = s - aH;
  h[kHdrShJ] = s - p.sy - aJ;
  h[kHdrShI] = s - p.sx - aI;
  h[kHdrJ] = jf;
  h[kHdrK] = f - jf * p.sy;
  h[kHdrCore] = i >= g.ilo && i < g.ihi && jf >= g.jlo && jl < g.jhi;
  constexpr uint32_t bytes = W * sizeof(float);
  float* d = ring + (size_t)st * g.nstream * W;
  // the arrival releases the header to the consumers that wait on this phase
  mbar_expect(bar, bytes * (uint32_t)g.nstream);
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
  for (int qq = 0; qq < 3 * NP; ++qq)
    bulk_copy(d + (kStT + qq) * W, T + (long long)qq * p.ncomp + aE, bytes, bar);
}

// One E node from a stage: the operands e_site loads from global memory, read from shared memory
// (S: the stage; shE, shH, shJ, shI: where node s of each stream group lies in its stream).
template <int PK, int NP, bool CORE, bool TR>
__device__ __forceinline__ void e_site_staged(const StepParams& p, const float4* C4, const float* Cs,
                                              const float2* CD, const float* __restrict__ S,
                                              int r, int shE, int shH, int shJ, int shI, int i,
                                              int j, int k, int idx, int it) {
  static_assert(NP == 0 || TR, "the staged sweep keeps real pole state only");
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
      t[comp][qq] = make_float2(sE[(kStT - kStE + comp * NP + qq) * W], 0.f);
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
  e_node<PK, NP, CORE, TR>(p, C4, Cs, CD, i, j, k, src, it, where, pr, hz_c - hz_j, hy_c - hy_k,
                           hx_c - hx_k, hz_c - hz_p, hy_c - hy_p, hx_c - hx_j, m, e, t);
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    p.E[comp][idx] = e[comp];
    if (disp) {
#pragma unroll
      for (int qq = 0; qq < NP; ++qq)
        reinterpret_cast<float*>(p.T)[(comp * NP + qq) * (long long)p.ncomp + idx] = t[comp][qq].x;
    }
  }
}

template <int PK, int NP, bool TR>
__global__ void __launch_bounds__(kStagedThreads, 1)
e_half_step_staged(const __grid_constant__ StepParams p, const __grid_constant__ StagedGeom g) {
  constexpr int W = kStageSpan;
  extern __shared__ __align__(128) float4 smem_st[];
  __shared__ uint64_t full[kStageMax], empty[kStageMax];
  __shared__ int hdr[kStageMax][kHdrInts];
  __shared__ int abort_flag;
  // after a sweep that gave up, the run's fields are void: later launches return at once, until
  // the host has read and cleared the error word
  if (*static_cast<volatile int*>(g.err)) return;
  float4* s4;
  float* ss;
  float2* sd;
  e_tables(p, smem_st, s4, ss, sd);
  float* ring = reinterpret_cast<float*>(reinterpret_cast<char*>(smem_st) + g.ring_off);
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
  stage_tables(p, true, s4, ss, NP > 0 ? sd : nullptr);
  __syncthreads();
  if (warp == 0) {
    // the producer: lane 0 fills the ring, a stage again once all consumer warps left it
    if (lane != 0) return;
    int n = 0;
    for (int c = blockIdx.x; c < g.nchunks; c += G, ++n) {
      const int st = n % g.nstages;
      if (n >= g.nstages &&
          !mbar_wait(&empty[st], (uint32_t)(n / g.nstages - 1) & 1u, g.limit_ns, abortp)) {
        *abortp = 1;
        atomicOr(g.err, 1);
        break;
      }
      // the consumers' reads of this stage are ordered before the copies that refill it
      proxy_async_fence();
      stage_chunk<NP>(p, g, ring, &full[st], hdr[st], c, st);
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
  const int it = p.nsrcE ? *p.d_it : 0;
  int n = 0;
  for (int c = blockIdx.x; c < g.nchunks; c += G, ++n) {
    const int st = n % g.nstages;
    if (!mbar_wait(&full[st], (uint32_t)(n / g.nstages) & 1u, g.limit_ns, abortp)) {
      *abortp = 1;
      atomicOr(g.err, 1);
      return;
    }
    const int* h = hdr[st];
    const int i = h[kHdrI], s = h[kHdrS];
    int j = h[kHdrJ] + tq, k = h[kHdrK] + tr;
    if (k >= p.sy) { k -= p.sy; ++j; }
    if (j >= 0 && j < p.ny && k < p.nz) {
      const float* S = ring + (size_t)st * g.nstream * W;
      if (h[kHdrCore])
        e_site_staged<PK, NP, true, TR>(p, s4, ss, sd, S, t, h[kHdrShE], h[kHdrShH], h[kHdrShJ],
                                        h[kHdrShI], i, j, k, s + t, it);
      else
        e_site_staged<PK, NP, false, TR>(p, s4, ss, sd, S, t, h[kHdrShE], h[kHdrShH],
                                         h[kHdrShJ], h[kHdrShI], i, j, k, s + t, it);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
  }
}

}  // namespace gbf
