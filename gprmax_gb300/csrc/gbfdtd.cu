// gbfdtd.cu — context, device memory, time loop and C ABI of libgbfdtd.so (see include/gbfdtd.h).
//
// Device layout (one allocation per array, all C order with k fastest):
//   fields   6 x fp32 [nx+1][ny+1][nz+1]         E then H; twice (two buffers) for models that
//                                                take the fused step, which reads one and writes
//                                                the other (ctx->cur is the current one)
//   ID       uint32 [6][nx+1][ny+1][nz+1]
//   T        float2 [3][P][nx+1][ny+1][nz+1]     dispersive state (P = maxpoles)
//   Phi      per slab, E and H, first and second tangential component, fp32 [order][...]
//            with layouts x:[p][j][k], y:[i][p][k], z:[i][j][p] (p = profile index)
//   rxs      fp32 [9][iterations][nrx]
// The iteration number lives in device memory and is advanced by the last kernel of each
// step, so a step is a fixed launch sequence that a CUDA graph can replay.
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbfdtd.h"
#include "fused_step.cuh"
#include "staged.cuh"

using namespace gbf;

// The device arrays that describe a model's materials (IDs, packed words, coefficient tables):
// owned by the context that uploaded them and shared by contexts that adopt them
// (gbf_share_materials); freed with the last context that holds them.
struct MatSet {
  std::vector<void*> ptrs;
  ~MatSet() {
    for (void* q : ptrs)
      if (q) cudaFree(q);
  }
};

struct gbf_ctx {
  gbf_grid_desc d;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long npts = 0;          // nodes per component, (nx+1)(ny+1)(nz+1)
  char* arena = nullptr;       // one allocation holding every array below but the material
                               // ones (ID, PE, PH, disp, tables: mats) and the snapshots
  long long ncomp = 0;         // device stride of one component array: npts rounded up to 64
                               // nodes, so every field, packed-ID and pole-state array starts
                               // on a 256-byte boundary (the staged E sweep copies them in
                               // 16-byte-aligned bulk copies)
  float* fields = nullptr;     // 6 * ncomp (12 * ncomp with the fused step's second buffer)
  uint32_t* ID = nullptr;      // 6 * npts, the caller's layout
  uint32_t* PE = nullptr;      // packed E IDs (ncomp), when nmat <= 1024
  uint32_t* PH = nullptr;      // packed H IDs
  unsigned char* disp = nullptr;   // per material: has dispersive poles
  int idp = 3;                 // 1: packed IDs, 3: three ID arrays per half-step
  int uniform_h = 0;           // every material has the same H row: the H half-step reads no IDs
  int treal = 0;               // T stored as fp32 real parts (Debye poles, packed IDs)
  float4* cE4 = nullptr;       // [nmat] CA, CBx, CBy, CBz
  float* cEs = nullptr;        // [nmat] srce
  float4* cH4 = nullptr;
  float* cHs = nullptr;
  size_t smem_e = 0, smem_h = 0;
  float2* cD = nullptr;
  float2* T = nullptr;
  float* pml_mem = nullptr;    // all Phi arrays
  float* pml_coef = nullptr;   // 6 slabs x (E,H) x [4][order][T]
  Src* srcs = nullptr;         // device: E sources in domain, H sources, E sources out of domain
  float* waves = nullptr;
  int* rx_coords = nullptr;
  float* rxs = nullptr;
  int* d_it = nullptr;
  TLine* tls = nullptr;        // transmission lines (device state)
  std::vector<TLine> tls_init; // their state at the start of the run
  float* tl_waves = nullptr;   // [ntl][2][iterations]
  float* tl_out = nullptr;     // [ntl][2][iterations]: Vtotal, Itotal
  std::vector<float*> snaps;
  std::vector<int> snapdef;    // nsnap x 10
  int it = 0;                  // host copy of the iteration counter
  bool materials = false;
  size_t bytes = 0;
  StepParams sp{};
  RxParams rp{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_steps = 0;
  int graph_cur = 0;           // field buffer current when the graph was captured
  int grid_h = 0, grid_e = 0;  // persistent grid sizes
  long long phi_floats = 0;    // all PML state (both H buffers for the fused step) and padding
  int zspan = 0;               // floats per z-slab Phi copy of the staged sweeps (0: no z slab)
  // fused step (fused_step.cuh): eligible models get two field buffers and two H PML buffers
  int fused_ok = 0;            // buffers allocated for it
  int fused_avail = 0;         // a fused kernel exists for the model (after the tables are known)
  int fused = 0;               // the step is the fused kernel (else the two half-step kernels)
  int cur = 0;                 // field / H PML buffer holding the current iteration
  float* phiH[6][2][2] = {};   // [slab][buffer][first/second component]
  FusedFn fk = nullptr;
  FusedTiles ft{};
  int f_tj = 0, f_blocks = 0;
  size_t smem_f = 0;
  int tuned = 0;
  std::vector<std::pair<int, int>> tune_cand;   // candidate (tile height, chunks) being timed
  std::vector<cudaEvent_t> tune_ev;             // two events per timed step
  int tune_next = 0;
  // staged half-steps (staged.cuh): used where they apply unless option bit 4 is set
  int staged = 0, staged_h = 0;       // the step's E / H half-step is the staged sweep
  int staged_av = 0;                  // where a staged sweep applies: bit 0 E, bit 1 H
  int forms_tuned = 1;                // staged or plain chosen (by the form tuner or the caller)
  std::vector<int> form_cand;         // combinations being timed (bit 0 staged E, bit 1 staged H)
  std::vector<cudaEvent_t> form_ev;   // two events per timed step
  int form_next = 0;
  SKernFn sk = nullptr, skh = nullptr;
  StagedGeom sg{}, sgh{};
  size_t smem_st = 0, smem_sth = 0;
  int* d_err = nullptr;        // device error word of the staged sweeps (a wait ran out)
  unsigned int* d_scr = nullptr;   // device scratch words: division check [0, 3), largest ID [4]
  std::shared_ptr<MatSet> mats;   // holds ID, PE, PH, disp and the tables (see MatSet)
  size_t mat_bytes = 0;        // their size
  bool shared_mats = false;    // adopted from another context
  bool dirty = false;          // the state may differ from the all-zero state it was created in
  bool ph_uploaded = true;     // the packed H words hold the model's H IDs (else zeros: every
                               // material has the same H row, and no kernel reads them)
};

static std::string g_create_err;
static void tune_release(gbf_ctx* ctx);
static void configure_staged(gbf_ctx* ctx);
static void form_release(gbf_ctx* ctx);
static bool form_cached(gbf_ctx* ctx);

static void invalidate_graph(gbf_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
}

static int fail(gbf_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf; else g_create_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA,          \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                        \
  } while (0)

static int dev_alloc(gbf_ctx* ctx, void** p, size_t n) {
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(p, n);
  if (e != cudaSuccess)
    return fail(ctx, GBF_ENOMEM, "cudaMalloc of %zu bytes failed: %s", n, cudaGetErrorString(e));
  ctx->bytes += n;
  CK(cudaMemsetAsync(*p, 0, n, ctx->stream));
  return GBF_OK;
}

// Does x/d computed as the corrected product with r = 1/d (div_cell in fdtd_kernels.cuh)
// equal the IEEE quotient for every x? The quotient's significand depends only on the
// significands of x and d while nothing leaves the normal range, and the kernel uses the
// product only for |x| in [2^-60, 2^80) with d in [2^-20, 2^20]; so one binade of x (all 2^23
// significands, positive; round-to-nearest is symmetric) decides it. Results are cached per d.
static bool reciprocal_division_exact(float d) {
  if (!(d >= 0x1p-20f && d <= 0x1p20f)) return false;
  static std::mutex mu;
  static std::vector<std::pair<uint32_t, bool>> cache;
  uint32_t bits;
  memcpy(&bits, &d, 4);
  {
    std::lock_guard<std::mutex> lock(mu);
    for (auto& c : cache)
      if (c.first == bits) return c.second;
  }
  const float r = 1.0f / d;
  // the 2^23 significands in slices over the host's cores, each slice without early exit
  unsigned nt = std::thread::hardware_concurrency();
  nt = nt < 1 ? 1 : (nt > 64 ? 64 : nt);
  std::vector<int> bad(nt, 0);
  auto slice = [&](unsigned t) {
    const uint32_t lo = (uint32_t)(((uint64_t)t << 23) / nt);
    const uint32_t hi = (uint32_t)(((uint64_t)(t + 1) << 23) / nt);
    int b = 0;
    for (uint32_t m = lo; m < hi; ++m) {
      const uint32_t xb = (127u << 23) | m;
      float x;
      memcpy(&x, &xb, 4);
      const float q = x * r;
      const float q1 = fmaf(fmaf(-q, d, x), r, q);
      b |= (q1 != x / d);
    }
    bad[t] = b;
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(slice, t);
  slice(0);
  for (auto& th : pool) th.join();
  bool ok = true;
  for (int b : bad) ok = ok && !b;
  std::lock_guard<std::mutex> lock(mu);
  cache.emplace_back(bits, ok);
  return ok;
}

// Sweep boxes of one half-step (Box in fdtd_kernels.cuh). Along x and y the domain splits into
// [0, lo), the core range [lo, hi) and [hi, end): E (end = n) has its minus slab at [1, Tm] and
// needs c >= 1 for every neighbour, so lo = Tm + 1; H (end = n + 1) has its minus slab at
// [0, Tm - 1] and needs c in [1, n - 1], so lo = max(Tm, 1); both have hi = n - Tp. Rows stay
// whole along z (the kernels test z-slab membership per node), so every box streams whole rows.
static void make_boxes(bool electric, const int n[3], const int T[6], Box out[kBoxes]) {
  int lo[3], hi[3], end[3];
  for (int a = 0; a < 3; ++a) {
    end[a] = electric ? n[a] : n[a] + 1;
    lo[a] = electric ? T[a] + 1 : (T[a] > 1 ? T[a] : 1);
    hi[a] = n[a] - T[a + 3];
    if (lo[a] > end[a]) lo[a] = end[a];
    if (hi[a] < lo[a]) hi[a] = lo[a];
  }
  auto box = [](int i0, int bi, int j0, int bj, int k0, int bk, int ksplit, int kgap) {
    Box b;
    b.i0 = i0; b.bi = bi; b.j0 = j0; b.bj = bj; b.k0 = k0; b.bk = bk;
    b.ksplit = ksplit; b.kgap = kgap;
    b.start = 0;
    b.count = (bi > 0 && bj > 0 && bk > 0) ? bi * bj * bk : 0;
    if (!b.count) b.bi = b.bj = b.bk = 1;   // keep the walker's divisors non-zero
    return b;
  };
  const int cx = hi[0] - lo[0], cy = hi[1] - lo[1], ez = end[2];
  out[0] = box(lo[0], cx, lo[1], cy, 0, ez, ez, 0);                           // core rows
  out[1] = box(0, lo[0], 0, end[1], 0, ez, ez, 0);                            // x minus planes
  out[2] = box(hi[0], end[0] - hi[0], 0, end[1], 0, ez, ez, 0);               // x plus planes
  out[3] = box(lo[0], cx, 0, lo[1], 0, ez, ez, 0);                            // y minus rows
  out[4] = box(lo[0], cx, hi[1], end[1] - hi[1], 0, ez, ez, 0);               // y plus rows
  out[5] = box(0, 0, 0, 0, 0, 0, 0, 0);                                       // unused
  int start = 0;
  for (int b = 0; b < kBoxes; ++b) {
    out[b].start = start;
    start += out[b].count;
  }
}

static int pml_kind(const gbf_grid_desc& d) {
  bool any = false;
  for (int s = 0; s < 6; ++s) any |= d.pml_thickness[s] > 0;
  if (!any) return PML_NONE;
  if (d.pml_formulation == GBF_PML_HORIPML) return d.pml_order == 1 ? PML_HORI1 : PML_HORI2;
  return d.pml_order == 1 ? PML_MRI1 : PML_MRI2;
}

// Point the kernel parameters at buffer `b` (fields and H PML state), which then holds the
// current iteration. En/Hn and phiH*n name the same arrays: the in-place form that every kernel
// but the fused step uses (the batch copies these parameters too).
static void set_current(gbf_ctx* ctx, int b) {
  ctx->cur = b;
  const long long n = ctx->ncomp;
  float* base = ctx->fields + (size_t)b * 6 * n;
  StepParams& p = ctx->sp;
  for (int c = 0; c < 3; ++c) {
    p.E[c] = p.En[c] = base + c * n;
    p.H[c] = p.Hn[c] = base + (3 + c) * n;
    ctx->rp.Eold[c] = p.E[c];
  }
  for (int s = 0; s < 6; ++s) {
    Slab& sl = p.slab[s];
    if (!sl.T) continue;
    sl.phiH1 = sl.phiH1n = ctx->phiH[s][b][0];
    sl.phiH2 = sl.phiH2n = ctx->phiH[s][b][1];
  }
}

static float* current_fields(const gbf_ctx* ctx) {
  return ctx->fields + (size_t)ctx->cur * 6 * ctx->ncomp;
}

// Parameters of a fused step that reads the current buffers and writes the other ones.
static StepParams fused_params(const gbf_ctx* ctx) {
  StepParams q = ctx->sp;
  const int o = ctx->cur ^ 1;
  const long long n = ctx->ncomp;
  float* base = ctx->fields + (size_t)o * 6 * n;
  for (int c = 0; c < 3; ++c) {
    q.En[c] = base + c * n;
    q.Hn[c] = base + (3 + c) * n;
  }
  for (int s = 0; s < 6; ++s) {
    Slab& sl = q.slab[s];
    if (!sl.T) continue;
    sl.phiH1n = ctx->phiH[s][o][0];
    sl.phiH2n = ctx->phiH[s][o][1];
  }
  return q;
}

// The launch decomposition for nch >= 1 chunks (clamped to [1, nx + 1]); nblocks < 0 when it
// does not fit.
static FusedTiles fused_tiles(int nx, int ny, int nz, int tj, int nch) {
  FusedTiles t;
  t.nseg = (nz + 1 + kTileK - 1) / kTileK;
  t.njt = (ny + 1 + tj - 1) / tj;
  const int planes = nx + 1;
  if (nch < 1) nch = 1;
  if (nch > planes) nch = planes;
  t.L = (planes + nch - 1) / nch;
  t.nch = (planes + t.L - 1) / t.L;
  const long long nw = (long long)t.nseg * t.njt * t.nch;
  t.nblocks = nw > (1LL << 30) ? -1 : (int)nw;
  return t;
}

static FusedFn fused_kernel(int pk, int tj, int np, int uh, int tr) {
  switch (tj * 10 + pk) {
    case 70: return fused_kernel_pk0_tj7(np, uh, tr);
    case 71: return fused_kernel_pk1_tj7(np, uh, tr);
    case 72: return fused_kernel_pk2_tj7(np, uh, tr);
    case 73: return fused_kernel_pk3_tj7(np, uh, tr);
    case 74: return fused_kernel_pk4_tj7(np, uh, tr);
    case 150: return fused_kernel_pk0_tj15(np, uh, tr);
    case 151: return fused_kernel_pk1_tj15(np, uh, tr);
    case 152: return fused_kernel_pk2_tj15(np, uh, tr);
    case 153: return fused_kernel_pk3_tj15(np, uh, tr);
    case 154: return fused_kernel_pk4_tj15(np, uh, tr);
    default: return nullptr;
  }
}

// The same question on the device for a model's three cell sizes at once (what gbf_create
// uses): bad[a] is set when the corrected product with r[a] differs from the IEEE quotient
// x / d[a] for some x of the binade [1, 2), computed with the kernels' own operations. The
// host loop takes about a millisecond per cell size; this takes microseconds.
__global__ void division_check(float3 d, float3 r, unsigned int* bad) {
  const int a = blockIdx.y;
  const float dd = a == 0 ? d.x : (a == 1 ? d.y : d.z);
  const float rr = a == 0 ? r.x : (a == 1 ? r.y : r.z);
  unsigned int b = 0;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < (1u << 23);
       m += gridDim.x * blockDim.x) {
    const float x = __uint_as_float((127u << 23) | m);
    const float q = __fmul_rn(x, rr);
    b |= __fmaf_rn(__fmaf_rn(-q, dd, x), rr, q) != __fdiv_rn(x, dd) ? 1u : 0u;
  }
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad + a, 1u);
}

// The device check's answers per cell size (bits of d; bad != 0: the product form is refused).
static std::mutex g_div_mu;
static std::vector<std::pair<uint32_t, unsigned int>> g_div;
static bool division_cached(float d, unsigned int& bad) {
  uint32_t bits;
  memcpy(&bits, &d, 4);
  std::lock_guard<std::mutex> lock(g_div_mu);
  for (auto& c : g_div)
    if (c.first == bits) {
      bad = c.second;
      return true;
    }
  return false;
}
static void division_remember(float d, unsigned int bad) {
  uint32_t bits;
  memcpy(&bits, &d, 4);
  std::lock_guard<std::mutex> lock(g_div_mu);
  for (auto& c : g_div)
    if (c.first == bits) return;
  g_div.emplace_back(bits, bad);
}

extern "C" {

const char* gbf_version(void) { return "gbfdtd 0.1 (sm_103a)"; }

int gbf_check_cell_division(float d) { return reciprocal_division_exact(d) ? 1 : 0; }

int gbf_check_cell_division_device(float d, int32_t* exact) {
  if (!exact) return fail(nullptr, GBF_EINVAL, "gbf_check_cell_division_device: NULL argument");
  *exact = 0;
  if (!(d >= 0x1p-20f && d <= 0x1p20f)) return GBF_OK;
  unsigned int* bad = nullptr;
  cudaError_t e = cudaMalloc((void**)&bad, 3 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(bad, 0, 3 * sizeof(unsigned int));
  if (e == cudaSuccess) {
    const float r = 1.0f / d;
    division_check<<<dim3(2048, 3), 256>>>(make_float3(d, d, d), make_float3(r, r, r), bad);
    e = cudaGetLastError();
  }
  unsigned int h[3] = {1u, 1u, 1u};
  if (e == cudaSuccess) e = cudaMemcpy(h, bad, sizeof h, cudaMemcpyDeviceToHost);
  if (bad) cudaFree(bad);
  if (e != cudaSuccess)
    return fail(nullptr, GBF_ECUDA, "gbf_check_cell_division_device: %s", cudaGetErrorString(e));
  *exact = (h[0] | h[1] | h[2]) ? 0 : 1;
  return GBF_OK;
}

int gbf_fused_tiles(int32_t nx, int32_t ny, int32_t nz, int32_t tj, int32_t nch, int32_t* out) {
  if (nx < 1 || ny < 1 || nz < 1 || tj < 1 || tj > 31 || !out) return GBF_EINVAL;
  const FusedTiles t = fused_tiles(nx, ny, nz, tj, nch);
  if (t.nblocks < 0) return GBF_EINVAL;
  const int32_t v[6] = {t.nseg, t.njt, t.nch, t.L, t.nblocks, kTileK};
  memcpy(out, v, sizeof v);
  return GBF_OK;
}

int gbf_sweep_boxes(int32_t nx, int32_t ny, int32_t nz, const int32_t thickness[6],
                    int32_t electric, int32_t* boxes) {
  if (nx < 1 || ny < 1 || nz < 1 || !thickness || !boxes) return GBF_EINVAL;
  for (int s = 0; s < 6; ++s)
    if (thickness[s] < 0 || 2 * thickness[s] >= (s % 3 == 0 ? nx : s % 3 == 1 ? ny : nz))
      return GBF_EINVAL;
  const int n[3] = {nx, ny, nz};
  Box b[kBoxes];
  make_boxes(electric != 0, n, thickness, b);
  for (int q = 0; q < kBoxes; ++q) {
    const int v[10] = {b[q].i0, b[q].j0, b[q].k0, b[q].bi, b[q].bj, b[q].bk, b[q].ksplit,
                       b[q].kgap, b[q].start, b[q].count};
    memcpy(boxes + 10 * q, v, sizeof(v));
  }
  return GBF_OK;
}

int gbf_last_error(gbf_ctx* ctx, char* buf, size_t n) {
  if (!buf || n == 0) return GBF_EINVAL;
  const std::string& s = ctx ? ctx->err : g_create_err;
  snprintf(buf, n, "%s", s.c_str());
  return GBF_OK;
}

void gbf_destroy(gbf_ctx* ctx) {
  if (!ctx) return;
  for (cudaEvent_t e : ctx->tune_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->form_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  if (ctx->arena) cudaFree(ctx->arena);
  // the material arrays go with the last context holding them
  ctx->mats.reset();
  for (float* p : ctx->snaps)
    if (p) cudaFree(p);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int gbf_create(const gbf_grid_desc* desc, gbf_ctx** out) {
  if (!desc || !out) return fail(nullptr, GBF_EINVAL, "gbf_create: NULL argument");
  *out = nullptr;
  const gbf_grid_desc& d = *desc;
  // 3D, or 2D with exactly one dimension of one cell (TMx, TMy, TMz)
  const int ones = (d.nx == 1) + (d.ny == 1) + (d.nz == 1);
  if (d.nx < 1 || d.ny < 1 || d.nz < 1 || ones > 1 ||
      (d.nx < 2 && d.nx != 1) || (d.ny < 2 && d.ny != 1) || (d.nz < 2 && d.nz != 1))
    return fail(nullptr, GBF_EINVAL, "gbf_create: grid must be 3D or 2D with one dimension of one cell (nx=%d ny=%d nz=%d)", d.nx, d.ny, d.nz);
  if (d.iterations < 1 || d.nmat < 1 || d.maxpoles < 0 || d.maxpoles > kMaxPoles)
    return fail(nullptr, GBF_EINVAL, "gbf_create: bad iterations/nmat/maxpoles (%d/%d/%d; poles <= %d)", d.iterations, d.nmat, d.maxpoles, kMaxPoles);
  if (d.pml_order < 1 || d.pml_order > 2 || (d.pml_formulation != 0 && d.pml_formulation != 1))
    return fail(nullptr, GBF_EINVAL, "gbf_create: PML order must be 1 or 2 and formulation 0 or 1");
  if (d.nsrc < 0 || d.nrx < 0 || d.nsnap < 0)
    return fail(nullptr, GBF_EINVAL, "gbf_create: negative counts");
  if ((d.options & ~63) || d.ntl < 0 || d.ntl > d.nsrc || d.reserved[0] || d.reserved[1])
    return fail(nullptr, GBF_EINVAL, "gbf_create: reserved fields must be zero");
  const long long npts = (long long)(d.nx + 1) * (d.ny + 1) * (d.nz + 1);
  if (npts + 63 > (1LL << 31) - 1)
    return fail(nullptr, GBF_EINVAL, "gbf_create: more than 2^31 - 64 nodes per component");
  const int n3[3] = {d.nx, d.ny, d.nz};
  for (int s = 0; s < 6; ++s) {
    const int t = d.pml_thickness[s];
    if (t < 0 || 2 * t >= n3[s % 3])
      return fail(nullptr, GBF_EINVAL, "gbf_create: PML slab %d thickness %d too large for the domain", s, t);
  }
  gbf_ctx* ctx = new gbf_ctx();
  ctx->d = d;
  ctx->npts = npts;
  ctx->ncomp = (npts + 63) & ~63LL;
  const long long ncomp = ctx->ncomp;
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    fail(nullptr, GBF_ECUDA, "gbf_create: CUDA unavailable: %s", cudaGetErrorString(e));
    delete ctx;
    return GBF_ECUDA;
  }
  // the fused step (3D, packed IDs, at most kFusedMaxPoles poles, no transmission lines, not
  // turned off by option bit 3) needs a second field buffer; without room for it the model
  // takes the two half-step kernels. With PML slabs the fused step is slower than the
  // half-step kernels and never chosen by timing, so such models get the second buffer only
  // when option bit 5 asks for it (to select the fused step with gbf_set_fused_tiles).
  bool any_pml = false;
  for (int s = 0; s < 6; ++s) any_pml |= d.pml_thickness[s] > 0;
  ctx->fused_ok = (ones == 0 && d.ntl == 0 && d.nmat <= 1024 && d.maxpoles <= kFusedMaxPoles &&
                   !(d.options & 8) && (!any_pml || (d.options & 32))) ? 1 : 0;
  // PML state: per slab 4 Phi arrays of order * T * nu * nv (6 with the second H buffer), each
  // starting on a 256-byte boundary; after them room for the staged sweeps' last z-slab copy,
  // which may read up to zspan floats past the end of an array
  auto phi_sum = [&](int nphi) {
    long long total = 0;
    for (int s = 0; s < 6; ++s) {
      const int t = d.pml_thickness[s];
      if (!t) continue;
      const int ax = s % 3;
      const long long nu = ax == 0 ? d.ny : d.nx, nv = ax == 2 ? d.ny : d.nz;
      total += (long long)nphi * ((d.pml_order * t * nu * nv + 63) & ~63LL);
    }
    return total;
  };
  const int tz = d.pml_thickness[2] > d.pml_thickness[5] ? d.pml_thickness[2] : d.pml_thickness[5];
  ctx->zspan = tz ? (int)((((kStageL + 2) / (d.nz + 1) + 2) * (long long)tz + 3 + 3) & ~3LL) : 0;
  int tmax = 1;
  for (int s = 0; s < 6; ++s) tmax = d.pml_thickness[s] > tmax ? d.pml_thickness[s] : tmax;
  // The state arrays in one allocation, cleared once, each on a 256-byte boundary (one
  // allocation instead of a score of them: creating a context is part of every model's upload)
  struct Carve {
    size_t off = 0;
    size_t take(size_t n) {
      const size_t o = off;
      off += (n + 255) & ~(size_t)255;
      return o;
    }
  };
  size_t o_fields = 0, o_T = 0, o_pml = 0, o_coef = 0, o_srcs = 0, o_waves = 0, o_rxc = 0,
         o_rxs = 0, o_it = 0, o_err = 0, o_scr = 0, o_tls = 0, o_tlw = 0, o_tlo = 0;
  auto layout = [&](bool two) {
    Carve c;
    o_fields = c.take(sizeof(float) * (two ? 12 : 6) * ncomp);
    if (d.maxpoles > 0) o_T = c.take(sizeof(float2) * 3 * (size_t)d.maxpoles * ncomp);
    ctx->phi_floats = phi_sum(two ? 6 : 4) + ctx->zspan + 64;
    o_pml = c.take(sizeof(float) * ctx->phi_floats);
    o_coef = c.take(sizeof(float) * 6 * 2 * 4 * d.pml_order * tmax);
    o_srcs = c.take(sizeof(Src) * (d.nsrc + 1));
    o_waves = c.take(sizeof(float) * (size_t)(d.nsrc + 1) * d.iterations);
    o_rxc = c.take(sizeof(int) * 3 * (d.nrx + 1));
    o_rxs = c.take(sizeof(float) * 9 * (size_t)d.iterations * (d.nrx + 1));
    o_it = c.take(sizeof(int));
    o_err = c.take(sizeof(int) * 16);
    o_scr = c.take(sizeof(unsigned int) * 16);
    if (d.ntl) {
      o_tls = c.take(sizeof(TLine) * d.ntl);
      o_tlw = c.take(sizeof(float) * 2 * (size_t)d.ntl * d.iterations);
      o_tlo = c.take(sizeof(float) * 2 * (size_t)d.ntl * d.iterations);
    }
    return c.off;
  };
  size_t total = layout(ctx->fused_ok != 0);
  cudaError_t me = cudaMalloc((void**)&ctx->arena, total);
  if (me != cudaSuccess && ctx->fused_ok) {
    // no room for the fused step's second buffers: the two half-step kernels do without
    (void)cudaGetLastError();
    ctx->fused_ok = 0;
    total = layout(false);
    me = cudaMalloc((void**)&ctx->arena, total);
  }
  int rc = GBF_OK;
  if (me != cudaSuccess) {
    (void)cudaGetLastError();
    ctx->arena = nullptr;
    rc = fail(ctx, GBF_ENOMEM, "gbf_create: cudaMalloc of %zu bytes failed: %s", total, cudaGetErrorString(me));
  } else {
    ctx->bytes += total;
    if (cudaMemsetAsync(ctx->arena, 0, total, ctx->stream) != cudaSuccess)
      rc = fail(ctx, GBF_ECUDA, "gbf_create: clearing the state failed");
    char* a = ctx->arena;
    ctx->fields = reinterpret_cast<float*>(a + o_fields);
    if (d.maxpoles > 0) ctx->T = reinterpret_cast<float2*>(a + o_T);
    ctx->pml_mem = reinterpret_cast<float*>(a + o_pml);
    ctx->pml_coef = reinterpret_cast<float*>(a + o_coef);
    ctx->srcs = reinterpret_cast<Src*>(a + o_srcs);
    ctx->waves = reinterpret_cast<float*>(a + o_waves);
    ctx->rx_coords = reinterpret_cast<int*>(a + o_rxc);
    ctx->rxs = reinterpret_cast<float*>(a + o_rxs);
    ctx->d_it = reinterpret_cast<int*>(a + o_it);
    ctx->d_err = reinterpret_cast<int*>(a + o_err);
    ctx->d_scr = reinterpret_cast<unsigned int*>(a + o_scr);
    if (d.ntl) {
      ctx->tls = reinterpret_cast<TLine*>(a + o_tls);
      ctx->tl_waves = reinterpret_cast<float*>(a + o_tlw);
      ctx->tl_out = reinterpret_cast<float*>(a + o_tlo);
    }
  }
  // The material arrays (packed IDs at most 1024 materials: two words per node, built
  // straight from the caller's array; otherwise the six ID arrays themselves; the coefficient
  // tables) in a second allocation, the one gbf_share_materials shares
  ctx->idp = d.nmat <= 1024 ? 1 : 3;
  Carve mc;
  const size_t o_pe = ctx->idp == 1 ? mc.take(sizeof(uint32_t) * ncomp) : 0;
  const size_t o_ph = ctx->idp == 1 ? mc.take(sizeof(uint32_t) * ncomp) : 0;
  const size_t o_id = ctx->idp == 1 ? 0 : mc.take(sizeof(uint32_t) * 6 * npts);
  const size_t o_disp = mc.take((size_t)d.nmat);
  const size_t o_ce4 = mc.take(sizeof(float4) * d.nmat);
  const size_t o_ces = mc.take(sizeof(float) * d.nmat);
  const size_t o_ch4 = mc.take(sizeof(float4) * d.nmat);
  const size_t o_chs = mc.take(sizeof(float) * d.nmat);
  const size_t o_cd = d.maxpoles > 0 ? mc.take(sizeof(float2) * 3 * d.maxpoles * d.nmat) : 0;
  char* m = nullptr;
  if (rc == GBF_OK) {
    me = cudaMalloc((void**)&m, mc.off);
    if (me != cudaSuccess) {
      (void)cudaGetLastError();
      m = nullptr;
      rc = fail(ctx, GBF_ENOMEM, "gbf_create: cudaMalloc of %zu bytes failed: %s", mc.off, cudaGetErrorString(me));
    } else if (cudaMemsetAsync(m, 0, mc.off, ctx->stream) != cudaSuccess) {
      rc = fail(ctx, GBF_ECUDA, "gbf_create: clearing the material arrays failed");
    }
  }
  if (m) {
    ctx->mats = std::make_shared<MatSet>();
    ctx->mats->ptrs = {m};
    ctx->mat_bytes = mc.off;
    ctx->bytes += mc.off;
    if (ctx->idp == 1) {
      ctx->PE = reinterpret_cast<uint32_t*>(m + o_pe);
      ctx->PH = reinterpret_cast<uint32_t*>(m + o_ph);
    } else {
      ctx->ID = reinterpret_cast<uint32_t*>(m + o_id);
    }
    ctx->disp = reinterpret_cast<unsigned char*>(m + o_disp);
    ctx->cE4 = reinterpret_cast<float4*>(m + o_ce4);
    ctx->cEs = reinterpret_cast<float*>(m + o_ces);
    ctx->cH4 = reinterpret_cast<float4*>(m + o_ch4);
    ctx->cHs = reinterpret_cast<float*>(m + o_chs);
    if (d.maxpoles > 0) ctx->cD = reinterpret_cast<float2*>(m + o_cd);
  }
  if (rc != GBF_OK) {
    g_create_err = ctx->err;
    gbf_destroy(ctx);
    return rc;
  }

  // kernel parameters
  StepParams& p = ctx->sp;
  for (int c = 0; c < 3; ++c) {
    p.E[c] = p.En[c] = ctx->fields + c * ncomp;
    p.H[c] = p.Hn[c] = ctx->fields + (3 + c) * ncomp;
  }
  for (int c = 0; c < 6; ++c) p.ID[c] = ctx->ID ? ctx->ID + c * npts : nullptr;
  p.PE = ctx->PE;
  p.PH = ctx->PH;
  for (int q = 0; q < kSrcInline; ++q) p.srcqE[q] = p.srcqH[q] = -1;
  p.ncomp = (int)ncomp;
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  p.two_d = (d.nx == 1 || d.ny == 1 || d.nz == 1) ? 1 : 0;
  p.sy = d.nz + 1;
  p.sx = (d.ny + 1) * (d.nz + 1);
  p.cE4 = ctx->cE4; p.cEs = ctx->cEs; p.cH4 = ctx->cH4; p.cHs = ctx->cHs;
  p.cD = ctx->cD; p.T = ctx->T; p.P = d.maxpoles;
  p.nmat = d.nmat;
  // shared-memory coefficient tables when they are small
  ctx->smem_h = (size_t)d.nmat * (sizeof(float4) + sizeof(float));
  ctx->smem_e = (size_t)d.nmat * sizeof(float4) + (size_t)((d.nmat + 3) & ~3) * sizeof(float) +
                (size_t)d.nmat * 3 * d.maxpoles * sizeof(float2);
  p.smem = (d.nmat <= kSmemCoefMax && ctx->smem_e <= 32768 && !(d.options & 1)) ? 1 : 0;
  if (!p.smem) ctx->smem_e = ctx->smem_h = 0;
  p.d_it = ctx->d_it;
  {
    const int n3b[3] = {d.nx, d.ny, d.nz};
    make_boxes(true, n3b, d.pml_thickness, p.boxE);
    make_boxes(false, n3b, d.pml_thickness, p.boxH);
  }
  float* phi = ctx->pml_mem;
  const float dd[3] = {d.dx, d.dy, d.dz};
  for (int s = 0; s < 6; ++s) {
    Slab& sl = p.slab[s];
    const int t = d.pml_thickness[s];
    sl.T = t;
    sl.d = dd[s % 3];
    sl.rcp = 1.0f / sl.d;
    // per axis (the kernels read it from the minus slab of either side's axis)
    const bool axis_pml = d.pml_thickness[s % 3] || d.pml_thickness[s % 3 + 3];
    // a candidate here; division_check below decides
    sl.fastdiv = (axis_pml && !(d.options & 2) && sl.d >= 0x1p-20f && sl.d <= 0x1p20f) ? 1 : 0;
    if (!t) continue;
    const int ax = s % 3;
    const long long nu = ax == 0 ? d.ny : d.nx, nv = ax == 2 ? d.ny : d.nz;
    sl.ocount = (int)(t * nu * nv);
    const long long per = ((long long)d.pml_order * sl.ocount + 63) & ~63LL;
    sl.phiE1 = phi; phi += per;
    sl.phiE2 = phi; phi += per;
    sl.phiH1 = phi; phi += per;
    sl.phiH2 = phi; phi += per;
    sl.phiH1n = sl.phiH1;
    sl.phiH2n = sl.phiH2;
    ctx->phiH[s][0][0] = ctx->phiH[s][1][0] = sl.phiH1;
    ctx->phiH[s][0][1] = ctx->phiH[s][1][1] = sl.phiH2;
    if (ctx->fused_ok) {
      ctx->phiH[s][1][0] = phi; phi += per;
      ctx->phiH[s][1][1] = phi; phi += per;
    }
    sl.eR = ctx->pml_coef + (size_t)(s * 2 + 0) * 4 * d.pml_order * tmax;
    sl.hR = ctx->pml_coef + (size_t)(s * 2 + 1) * 4 * d.pml_order * tmax;
  }
  p.nsrcE = p.nsrcH = 0;
  p.srcE = p.srcH = ctx->srcs;
  RxParams& r = ctx->rp;
  for (int c = 0; c < 3; ++c) r.Eold[c] = p.E[c];
  r.coords = ctx->rx_coords;
  r.out = ctx->rxs;
  r.nrx = d.nrx;
  r.iterations = d.iterations;
  r.dx = d.dx; r.dy = d.dy; r.dz = d.dz;
  r.nsrcOut = 0;
  r.srcOut = ctx->srcs;
  r.tls = ctx->tls;
  r.ntl = 0;
  r.tl_out = ctx->tl_out;
  // the corrected-product division per axis, checked on the device (after the arena's clear,
  // which zeroes the flags)
  // (answers kept per cell size for the process: a B-scan's models ask it once)
  if (p.slab[0].fastdiv || p.slab[1].fastdiv || p.slab[2].fastdiv) {
    unsigned int bad[3] = {1u, 1u, 1u};
    bool known = true;
    for (int a = 0; a < 3; ++a)
      if (p.slab[a].fastdiv) known = known && division_cached(p.slab[a].d, bad[a]);
    if (!known) {
      division_check<<<dim3(2048, 3), 256, 0, ctx->stream>>>(
          make_float3(p.slab[0].d, p.slab[1].d, p.slab[2].d),
          make_float3(p.slab[0].rcp, p.slab[1].rcp, p.slab[2].rcp), ctx->d_scr);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(bad, ctx->d_scr, sizeof bad, cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e == cudaSuccess)
        for (int a = 0; a < 3; ++a)
          if (p.slab[a].fastdiv) division_remember(p.slab[a].d, bad[a]);
    }
    for (int s = 0; s < 6; ++s) p.slab[s].fastdiv = p.slab[s].fastdiv && !bad[s % 3];
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    fail(nullptr, GBF_ECUDA, "gbf_create: %s", cudaGetErrorString(e));
    gbf_destroy(ctx);
    return GBF_ECUDA;
  }
  *out = ctx;
  return GBF_OK;
}

}  // extern "C"

// Let kernel k take `need` bytes of dynamic shared memory. The limit belongs to the kernel, not
// to a context, and every launch states its own size; so the limit is raised once to all the
// device allows beside the kernel's static shared memory, and never lowered by a context that
// needs less (contexts of different sizes may launch the same kernel in any order, as a batch
// does).
static bool allow_dynamic_smem(const void* k, size_t need, int device) {
  cudaFuncAttributes a{};
  if (cudaFuncGetAttributes(&a, k) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if ((size_t)a.maxDynamicSharedSizeBytes >= need) return true;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  const long long most = (long long)optin - (long long)a.sharedSizeBytes;
  if ((long long)need > most ||
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return true;
}

// Tiles of the fused step: k segments of kTileK nodes, j tiles of `tj` rows and `nch` chunks of
// planes along x (nch <= 0: as many chunks as give one wave of resident warps). Returns 0 when
// no fused kernel exists for the model or the tiling does not fit.
static int configure_fused(gbf_ctx* ctx, int tj, int nch) {
  const gbf_grid_desc& d = ctx->d;
  FusedFn f = fused_kernel(pml_kind(d), tj, d.maxpoles, ctx->uniform_h, ctx->treal);
  if (!f) return 0;
  size_t sm = 0;
  if (ctx->sp.smem) sm = ctx->smem_e + 16 + (ctx->uniform_h ? 0 : ctx->smem_h);
  if (sm > 48 * 1024 && !allow_dynamic_smem((const void*)f, sm, ctx->device)) return 0;
  if (nch <= 0) {   // one wave of resident warps
    const FusedTiles one = fused_tiles(d.nx, d.ny, d.nz, tj, 1);
    int dev = 0, sms = 1, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)f, (tj + 1) * 32, sm);
    const long long resident = (long long)sms * (per > 0 ? per : 1);
    nch = (int)(resident / ((long long)one.nseg * one.njt));
  }
  const FusedTiles t = fused_tiles(d.nx, d.ny, d.nz, tj, nch);
  if (t.nblocks < 0) return 0;
  ctx->fk = f;
  ctx->ft = t;
  ctx->f_tj = tj;
  ctx->smem_f = sm;
  ctx->f_blocks = t.nblocks;
  return 1;
}

// Packed per-node material words (IDs < 1024) from an ID array [6][n] that the device can read
// (device memory, or host memory the device reaches directly or through a mapping): E word the
// Ex, Ey, Ez IDs and bit 30 when one of them has dispersive poles, H word the Hx, Hy, Hz IDs.
// The largest ID goes to *mx, so that one pass both packs and checks the array.
__global__ void pack_ids_from(const uint32_t* __restrict__ ID, long long n, int nmat,
                              const unsigned char* __restrict__ disp, uint32_t* __restrict__ pe,
                              uint32_t* __restrict__ ph, unsigned int* mx) {
  unsigned int m = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const uint32_t ex = ID[q], ey = ID[n + q], ez = ID[2 * n + q];
    const uint32_t hx = ID[3 * n + q], hy = ID[4 * n + q], hz = ID[5 * n + q];
    const uint32_t a = max(max(ex, ey), ez), b = max(max(hx, hy), hz);
    m = max(m, max(a, b));
    uint32_t w = (ex & kPackMask) | ((ey & kPackMask) << kPackBits) | ((ez & kPackMask) << (2 * kPackBits));
    if (disp && a < (uint32_t)nmat && (disp[ex] | disp[ey] | disp[ez])) w |= kDispersiveBit;
    pe[q] = w;
    ph[q] = (hx & kPackMask) | ((hy & kPackMask) << kPackBits) | ((hz & kPackMask) << (2 * kPackBits));
  }
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// Packed words copied in as the caller packed them (gbf_pack_ids: no dispersive flag): add the
// flag to the E words and put the largest ID in *mx.
__global__ void finish_packed_ids(uint32_t* __restrict__ pe, const uint32_t* __restrict__ ph,
                                  long long n, int nmat, const unsigned char* __restrict__ disp,
                                  unsigned int* mx) {
  unsigned int m = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    uint32_t w = pe[q];
    const uint32_t h = ph ? ph[q] : 0u;
    const uint32_t ex = w & kPackMask, ey = (w >> kPackBits) & kPackMask, ez = (w >> (2 * kPackBits)) & kPackMask;
    const uint32_t a = max(max(ex, ey), ez);
    const uint32_t b = max(max(h & kPackMask, (h >> kPackBits) & kPackMask), (h >> (2 * kPackBits)) & kPackMask);
    m = max(m, max(a, b));
    if (w >> (3 * kPackBits)) m = 0xffffffffu;   // bits above the three IDs must be clear
    if (disp && a < (uint32_t)nmat && (disp[ex] | disp[ey] | disp[ez])) pe[q] = w | kDispersiveBit;
  }
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// Once the model's material tables are known: how it steps (fused step, staged half-steps) and
// whether those choices are still to be timed.
static void configure_steps(gbf_ctx* ctx) {
  ctx->grid_h = 0;
  ctx->grid_e = 0;
  invalidate_graph(ctx);
  // one fused kernel per step where the model allows it (tiles tuned at the first run)
  tune_release(ctx);
  ctx->fused_avail = ctx->fused_ok ? configure_fused(ctx, 7, 0) : 0;
  // measured on the GB300: with PML slabs the fused step runs slower than the two half-step
  // kernels (its slab nodes wait on their PML state within each plane), so such models take the
  // half-step kernels without timing the fused one (gbf_set_fused_tiles still selects it)
  const bool timed = ctx->fused_avail && pml_kind(ctx->d) == PML_NONE;
  ctx->fused = timed ? 1 : 0;
  ctx->tuned = timed ? 0 : 1;
  // GBF_FUSED_TILE="tj,nch" selects the fused step with that tiling for every model that has one
  const char* force = getenv("GBF_FUSED_TILE");
  int ftj = 0, fnch = 0;
  if (ctx->fused_avail && force && sscanf(force, "%d,%d", &ftj, &fnch) == 2 &&
      configure_fused(ctx, ftj, fnch)) {
    ctx->fused = 1;
    ctx->tuned = 1;
  }
  // the staged half-steps and whether their form is still to be chosen
  configure_staged(ctx);
}

// Coefficient tables, dispersive flags and, with packed IDs, the packed words: from `ids` (an ID
// array [6][ncomp] the device can read), or, with `ids` NULL, from the words already copied into
// ctx->PE/PH by the caller's packing. Plain IDs are already in ctx->ID.
static int upload_tables(gbf_ctx* ctx, const float* coeffE, const float* coeffH,
                         const float* coeffD, const uint32_t* ids) {
  const int nmat = ctx->d.nmat;
  // one H row for every material (no magnetic materials): the H half-step then needs no IDs
  int uni = 1;
  for (int m = 1; m < nmat && uni; ++m)
    uni = memcmp(coeffH + 5 * m, coeffH, 5 * sizeof(float)) == 0;
  ctx->uniform_h = uni;
  // the shared row, read from the kernel parameters by the ID-free H half-step
  for (int q = 0; q < 5; ++q) ctx->sp.hrow[q] = coeffH[q];
  ctx->sp.hrow[5] = 0.f;
  // real dispersive state: every pole's eqt has imaginary part +0 and zt imaginary part +-0
  // (Debye poles; the E update reads only Re(T), and Im(T) then stays +0), packed IDs, and the
  // complex layout not requested (option bit 2)
  int tr = ctx->d.maxpoles > 0 && ctx->idp == 1 && !(ctx->d.options & 4);
  for (int m = 0; m < nmat && tr; ++m)
    for (int q = 0; q < ctx->d.maxpoles && tr; ++q) {
      const float* c = coeffD + ((size_t)m * 3 * ctx->d.maxpoles + 3 * q) * 2;
      uint32_t eqt_im, zt_im;
      memcpy(&eqt_im, c + 3, 4);
      memcpy(&zt_im, c + 5, 4);
      tr = eqt_im == 0u && (zt_im & 0x7fffffffu) == 0u;
    }
  if (tr != ctx->treal && ctx->T) {
    // the layout changes: start the state again from zero
    CK(cudaMemsetAsync(ctx->T, 0, sizeof(float2) * 3 * (size_t)ctx->d.maxpoles * ctx->ncomp, ctx->stream));
  }
  ctx->treal = tr;
  configure_steps(ctx);
  std::vector<float4> e4(nmat), h4(nmat);
  std::vector<float> es(nmat), hs(nmat);
  for (int m = 0; m < nmat; ++m) {
    const float* a = coeffE + 5 * m;
    const float* b = coeffH + 5 * m;
    e4[m] = make_float4(a[0], a[1], a[2], a[3]);
    es[m] = a[4];
    h4[m] = make_float4(b[0], b[1], b[2], b[3]);
    hs[m] = b[4];
  }
  CK(cudaMemcpyAsync(ctx->cE4, e4.data(), sizeof(float4) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->cEs, es.data(), sizeof(float) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->cH4, h4.data(), sizeof(float4) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->cHs, hs.data(), sizeof(float) * nmat, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<unsigned char> disp(nmat, 0);
  if (ctx->d.maxpoles > 0 && tr) {
    // real pole state: one record per material and pole, (Re(e0*eqt2), Re(eqt), Re(zt), srce),
    // in the space of the complex table
    const int P = ctx->d.maxpoles;
    std::vector<float4> rec((size_t)nmat * P);
    for (int m = 0; m < nmat; ++m)
      for (int q = 0; q < P; ++q) {
        const float* c = coeffD + ((size_t)m * 3 * P + 3 * q) * 2;
        rec[(size_t)m * P + q] = make_float4(c[0], c[2], c[4], coeffE[5 * m + 4]);
      }
    CK(cudaMemcpyAsync(ctx->cD, rec.data(), sizeof(float4) * rec.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
  } else if (ctx->d.maxpoles > 0) {
    CK(cudaMemcpyAsync(ctx->cD, coeffD, sizeof(float2) * 3 * ctx->d.maxpoles * nmat,
                       cudaMemcpyHostToDevice, ctx->stream));
  }
  if (ctx->d.maxpoles > 0) {
    for (int m = 0; m < nmat; ++m)
      for (int q = 0; q < 6 * ctx->d.maxpoles; ++q)
        if (coeffD[(size_t)m * 6 * ctx->d.maxpoles + q] != 0.f) disp[m] = 1;
  }
  CK(cudaMemcpyAsync(ctx->disp, disp.data(), nmat, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->idp == 1) {
    unsigned int* dmax = ctx->d_scr + 4;
    CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned int), ctx->stream));
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ids) ctx->ph_uploaded = true;
    if (ids)
      pack_ids_from<<<sms * 8, 256, 0, ctx->stream>>>(ids, ctx->npts, nmat,
                                                     ctx->d.maxpoles > 0 ? ctx->disp : nullptr,
                                                     ctx->PE, ctx->PH, dmax);
    else
      finish_packed_ids<<<sms * 8, 256, 0, ctx->stream>>>(ctx->PE, ctx->ph_uploaded ? ctx->PH : nullptr,
                                                         ctx->npts, nmat,
                                                         ctx->d.maxpoles > 0 ? ctx->disp : nullptr,
                                                         dmax);
    CK(cudaGetLastError());
    unsigned int mx = 0;
    CK(cudaMemcpyAsync(&mx, dmax, sizeof mx, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (mx >= (unsigned)nmat) {
      ctx->materials = false;
      if (mx == 0xffffffffu)
        return fail(ctx, GBF_EINVAL, "packed material words have bits set above the three IDs");
      return fail(ctx, GBF_EINVAL, "material ID %u >= nmat %d", mx, nmat);
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->materials = true;
  return GBF_OK;
}

namespace gbf {
const uint32_t* geom_ids(const gbf_geom* g, int dims[3], int* device, cudaStream_t* stream);
}

__global__ void id_max_kernel(const uint32_t* a, long long n, unsigned int* mx) {
  unsigned int m = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    m = a[q] > m ? a[q] : m;
  for (int o = 16; o; o >>= 1) {
    const unsigned int t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// The largest ID in ctx->ID (on the device) must index the coefficient tables.
static int check_ids(gbf_ctx* ctx, const char* who) {
  const size_t n = 6 * (size_t)ctx->npts;
  unsigned int* dmax = ctx->d_scr + 4;
  CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned int), ctx->stream));
  id_max_kernel<<<1024, 256, 0, ctx->stream>>>(ctx->ID, (long long)n, dmax);
  CK(cudaGetLastError());
  unsigned int mx = 0;
  CK(cudaMemcpyAsync(&mx, dmax, sizeof mx, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (mx >= (unsigned)ctx->d.nmat)
    return fail(ctx, GBF_EINVAL, "%s: ID %u >= nmat %d", who, mx, ctx->d.nmat);
  return GBF_OK;
}

extern "C" {

int gbf_upload_materials(gbf_ctx* ctx, const uint32_t* ID, const float* coeffE,
                         const float* coeffH, const float* coeffD) {
  if (!ctx) return GBF_EINVAL;
  if (!ID || !coeffE || !coeffH || (ctx->d.maxpoles > 0 && !coeffD))
    return fail(ctx, GBF_EINVAL, "gbf_upload_materials: NULL array");
  const size_t n = 6 * (size_t)ctx->npts;
  const size_t bytes = sizeof(uint32_t) * n;
  if (ctx->idp == 1) {
    // packed IDs: one kernel reads the caller's array where it lies and writes the two words
    // per node, checking every ID on the way. Where the device reads pageable host memory
    // through the host's page tables (NVLink-C2C systems) it reads the array directly; else the
    // array is page-locked and mapped for the kernel, or, where that is refused, copied to a
    // device buffer first. The array is not kept on the device.
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, ctx->device);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device);
    const uint32_t* src = nullptr;
    bool mapped = false;
    uint32_t* tmp = nullptr;
    if (pageable && host_tables) {
      src = ID;
    } else if (cudaHostRegister(const_cast<uint32_t*>(ID), bytes,
                                cudaHostRegisterMapped | cudaHostRegisterReadOnly) == cudaSuccess) {
      mapped = true;
      void* dp = nullptr;
      if (cudaHostGetDevicePointer(&dp, const_cast<uint32_t*>(ID), 0) == cudaSuccess) {
        src = static_cast<const uint32_t*>(dp);
      } else {
        (void)cudaGetLastError();
      }
    } else {
      (void)cudaGetLastError();
    }
    if (!src) {
      if (cudaMalloc((void**)&tmp, bytes) != cudaSuccess) {
        if (mapped) cudaHostUnregister(const_cast<uint32_t*>(ID));
        return fail(ctx, GBF_ENOMEM, "gbf_upload_materials: no room for the ID array");
      }
      cudaError_t ce = cudaMemcpyAsync(tmp, ID, bytes, cudaMemcpyHostToDevice, ctx->stream);
      if (ce != cudaSuccess) {
        cudaFree(tmp);
        if (mapped) cudaHostUnregister(const_cast<uint32_t*>(ID));
        return fail(ctx, GBF_ECUDA, "gbf_upload_materials: ID copy: %s", cudaGetErrorString(ce));
      }
      src = tmp;
    }
    const int rc = upload_tables(ctx, coeffE, coeffH, coeffD, src);   // synchronises the stream
    if (tmp) cudaFree(tmp);
    if (mapped) cudaHostUnregister(const_cast<uint32_t*>(ID));
    return rc;
  }
  // plain IDs: a large array is page-locked for the copy (registration is cheap next to the
  // first copy of pageable memory); where that is refused the copy goes from pageable memory
  bool locked = false;
  if (bytes >= ((size_t)64 << 20)) {
    locked = cudaHostRegister(const_cast<uint32_t*>(ID), bytes, cudaHostRegisterReadOnly) == cudaSuccess;
    if (!locked) (void)cudaGetLastError();
  }
  cudaError_t ce = cudaMemcpyAsync(ctx->ID, ID, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (locked) {
    cudaError_t se = cudaStreamSynchronize(ctx->stream);
    cudaHostUnregister(const_cast<uint32_t*>(ID));
    if (ce == cudaSuccess) ce = se;
  }
  if (ce != cudaSuccess)
    return fail(ctx, GBF_ECUDA, "gbf_upload_materials: ID copy: %s", cudaGetErrorString(ce));
  // every ID must index the tables (checked on the device)
  const int rc = check_ids(ctx, "gbf_upload_materials");
  if (rc != GBF_OK) return rc;
  return upload_tables(ctx, coeffE, coeffH, coeffD, nullptr);
}

int gbf_upload_materials_packed(gbf_ctx* ctx, const uint32_t* PE, const uint32_t* PH,
                                const float* coeffE, const float* coeffH, const float* coeffD) {
  if (!ctx) return GBF_EINVAL;
  if (!PE || !coeffE || !coeffH || (ctx->d.maxpoles > 0 && !coeffD))
    return fail(ctx, GBF_EINVAL, "gbf_upload_materials_packed: NULL array");
  // the H words may be left out when every material has the same H row: no kernel reads them
  if (!PH)
    for (int m = 1; m < ctx->d.nmat; ++m)
      if (memcmp(coeffH + 5 * m, coeffH, 5 * sizeof(float)) != 0)
        return fail(ctx, GBF_EINVAL, "gbf_upload_materials_packed: the H words may be omitted only "
                    "when every material has the same H row (material %d differs)", m);
  if (ctx->idp != 1)
    return fail(ctx, GBF_EINVAL, "gbf_upload_materials_packed: %d materials do not pack (at most 1024)", ctx->d.nmat);
  const size_t bytes = sizeof(uint32_t) * (size_t)ctx->npts;
  CK(cudaMemcpyAsync(ctx->PE, PE, bytes, cudaMemcpyHostToDevice, ctx->stream));
  if (PH) CK(cudaMemcpyAsync(ctx->PH, PH, bytes, cudaMemcpyHostToDevice, ctx->stream));
  ctx->ph_uploaded = PH != nullptr;
  return upload_tables(ctx, coeffE, coeffH, coeffD, nullptr);
}

int gbf_pack_ids(const uint32_t* ID, int64_t n, uint32_t* PE, uint32_t* PH, uint32_t* maxid) {
  if (!ID || !PE || n < 1) return fail(nullptr, GBF_EINVAL, "gbf_pack_ids: bad arguments");
  // contiguous ranges over the host's cores; each range packs and keeps its largest ID
  unsigned nt = std::thread::hardware_concurrency();
  nt = nt < 1 ? 1 : (nt > 64 ? 64 : nt);
  if ((int64_t)nt > n / 65536 + 1) nt = (unsigned)(n / 65536 + 1);
  std::vector<uint32_t> mx(nt, 0);
  auto work = [&](unsigned t) {
    const int64_t lo = n * (int64_t)t / nt, hi = n * (int64_t)(t + 1) / nt;
    uint32_t m = 0;
    if (PH) {
      for (int64_t q = lo; q < hi; ++q) {
        const uint32_t ex = ID[q], ey = ID[n + q], ez = ID[2 * n + q];
        const uint32_t hx = ID[3 * n + q], hy = ID[4 * n + q], hz = ID[5 * n + q];
        const uint32_t a = ex > ey ? ex : ey, b = hx > hy ? hx : hy;
        const uint32_t c = ez > hz ? ez : hz;
        const uint32_t ab = a > b ? a : b;
        m = m > ab ? m : ab;
        m = m > c ? m : c;
        PE[q] = (ex & kPackMask) | ((ey & kPackMask) << kPackBits) | ((ez & kPackMask) << (2 * kPackBits));
        PH[q] = (hx & kPackMask) | ((hy & kPackMask) << kPackBits) | ((hz & kPackMask) << (2 * kPackBits));
      }
    } else {
      // the E words only (a model whose materials share one H row needs no H IDs)
      for (int64_t q = lo; q < hi; ++q) {
        const uint32_t ex = ID[q], ey = ID[n + q], ez = ID[2 * n + q];
        const uint32_t a = ex > ey ? ex : ey;
        m = m > a ? m : a;
        m = m > ez ? m : ez;
        PE[q] = (ex & kPackMask) | ((ey & kPackMask) << kPackBits) | ((ez & kPackMask) << (2 * kPackBits));
      }
    }
    mx[t] = m;
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  uint32_t m = 0;
  for (uint32_t v : mx) m = m > v ? m : v;
  if (maxid) *maxid = m;
  if (m > kPackMask) return fail(nullptr, GBF_EINVAL, "gbf_pack_ids: material ID %u does not fit 10 bits", m);
  return GBF_OK;
}

int gbf_host_alloc(size_t bytes, void** out) {
  if (!out) return GBF_EINVAL;
  *out = nullptr;
  cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail(nullptr, e == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA,
                "gbf_host_alloc: %s", cudaGetErrorString(e));
  }
  return GBF_OK;
}

void gbf_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int gbf_upload_materials_geom(gbf_ctx* ctx, gbf_geom* geom, const float* coeffE,
                              const float* coeffH, const float* coeffD) {
  if (!ctx) return GBF_EINVAL;
  if (!geom || !coeffE || !coeffH || (ctx->d.maxpoles > 0 && !coeffD))
    return fail(ctx, GBF_EINVAL, "gbf_upload_materials_geom: NULL argument");
  int dims[3], gdev = -1;
  cudaStream_t gstream = nullptr;
  const uint32_t* gid = geom_ids(geom, dims, &gdev, &gstream);
  if (dims[0] != ctx->d.nx || dims[1] != ctx->d.ny || dims[2] != ctx->d.nz || gdev != ctx->device)
    return fail(ctx, GBF_EINVAL, "gbf_upload_materials_geom: geometry %d x %d x %d on device %d "
                "does not match the context's grid %d x %d x %d on device %d", dims[0], dims[1],
                dims[2], gdev, ctx->d.nx, ctx->d.ny, ctx->d.nz, ctx->device);
  const size_t n = 6 * (size_t)ctx->npts;
  CK(cudaStreamSynchronize(gstream));
  if (ctx->idp == 1)   // packed straight from the geometry's IDs
    return upload_tables(ctx, coeffE, coeffH, coeffD, gid);
  CK(cudaMemcpyAsync(ctx->ID, gid, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  const int rc = check_ids(ctx, "gbf_upload_materials_geom");
  if (rc != GBF_OK) return rc;
  return upload_tables(ctx, coeffE, coeffH, coeffD, nullptr);
}

int gbf_share_materials(gbf_ctx* ctx, gbf_ctx* owner) {
  if (!ctx) return GBF_EINVAL;
  if (!owner || owner == ctx) return fail(ctx, GBF_EINVAL, "gbf_share_materials: no other context given");
  if (!owner->materials)
    return fail(ctx, GBF_ESTATE, "gbf_share_materials: the other context has no materials uploaded");
  const gbf_grid_desc& a = ctx->d;
  const gbf_grid_desc& b = owner->d;
  if (a.nx != b.nx || a.ny != b.ny || a.nz != b.nz || a.nmat != b.nmat ||
      a.maxpoles != b.maxpoles || (a.options & 4) != (b.options & 4) || ctx->device != owner->device)
    return fail(ctx, GBF_EINVAL, "gbf_share_materials: grids, material counts, pole counts, the "
                "dispersive-state layout (options bit 2) and devices must be the same");
  CK(cudaStreamSynchronize(owner->stream));
  // this context's own material arrays go (with the last context that holds them)
  if (!ctx->shared_mats) ctx->bytes -= ctx->mat_bytes;
  ctx->mats = owner->mats;
  ctx->shared_mats = true;
  ctx->ID = owner->ID;
  ctx->PE = owner->PE;
  ctx->PH = owner->PH;
  ctx->disp = owner->disp;
  ctx->cE4 = owner->cE4;
  ctx->cEs = owner->cEs;
  ctx->cH4 = owner->cH4;
  ctx->cHs = owner->cHs;
  ctx->cD = owner->cD;
  ctx->idp = owner->idp;
  ctx->uniform_h = owner->uniform_h;
  if (owner->treal != ctx->treal && ctx->T)
    CK(cudaMemsetAsync(ctx->T, 0, sizeof(float2) * 3 * (size_t)a.maxpoles * ctx->ncomp, ctx->stream));
  ctx->treal = owner->treal;
  StepParams& p = ctx->sp;
  const StepParams& q = owner->sp;
  for (int c = 0; c < 6; ++c) p.ID[c] = q.ID[c];
  p.PE = q.PE;
  p.PH = q.PH;
  p.cE4 = q.cE4;
  p.cEs = q.cEs;
  p.cH4 = q.cH4;
  p.cHs = q.cHs;
  p.cD = q.cD;
  for (int k = 0; k < 6; ++k) p.hrow[k] = q.hrow[k];
  configure_steps(ctx);
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->materials = true;
  return GBF_OK;
}

int gbf_upload_pml(gbf_ctx* ctx, int slab, const float* const rows[8]) {
  if (!ctx) return GBF_EINVAL;
  if (slab < 0 || slab >= 6 || !rows) return fail(ctx, GBF_EINVAL, "gbf_upload_pml: bad slab %d", slab);
  const int t = ctx->d.pml_thickness[slab];
  if (!t) return fail(ctx, GBF_EINVAL, "gbf_upload_pml: slab %d has zero thickness", slab);
  int tmax = 1;
  for (int s = 0; s < 6; ++s) tmax = ctx->d.pml_thickness[s] > tmax ? ctx->d.pml_thickness[s] : tmax;
  const int order = ctx->d.pml_order;
  // rows are [order][thickness]; device rows [q][order][T] with T == thickness: the four rows
  // of each field type gathered on the host and copied at once
  std::vector<float> four((size_t)4 * order * t);
  for (int h = 0; h < 2; ++h) {
    float* base = ctx->pml_coef + (size_t)(slab * 2 + h) * 4 * order * tmax;
    for (int q = 0; q < 4; ++q) {
      const float* src = rows[h * 4 + q];
      if (!src) return fail(ctx, GBF_EINVAL, "gbf_upload_pml: NULL row");
      memcpy(four.data() + (size_t)q * order * t, src, sizeof(float) * order * t);
    }
    // a copy from pageable memory is staged before the call returns, so `four` may be reused
    // at once; the stream is synchronised later (gbf_reset, gbf_synchronize, the first run)
    CK(cudaMemcpyAsync(base, four.data(), sizeof(float) * four.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  return GBF_OK;
}

int gbf_upload_sources(gbf_ctx* ctx, const int32_t* info, const float* scale, const float* waves) {
  if (!ctx) return GBF_EINVAL;
  const gbf_grid_desc& d = ctx->d;
  if (d.nsrc == 0) return GBF_OK;
  if (!info || !scale || !waves) return fail(ctx, GBF_EINVAL, "gbf_upload_sources: NULL array");
  std::vector<Src> inE, inH, outE;
  int ntl_seen = 0;
  for (int s = 0; s < d.nsrc; ++s) {
    const int32_t* q = info + 8 * s;
    Src v{};
    v.kind = q[0]; v.comp = q[1]; v.i = q[2]; v.j = q[3]; v.k = q[4];
    v.first = q[5]; v.last = q[6];
    v.s0 = scale[2 * s]; v.s1 = scale[2 * s + 1];
    v.w = ctx->waves + (size_t)s * d.iterations;
    if (v.kind == GBF_SRC_TRANSMISSION_LINE) {
      // the E half-step reads the line's -V/d; lines are numbered in source order
      if (ntl_seen >= d.ntl)
        return fail(ctx, GBF_EINVAL, "gbf_upload_sources: more transmission lines than desc.ntl");
      v.w = &ctx->tls[ntl_seen].eset;
      ++ntl_seen;
    }
    if (v.kind < 0 || v.kind > 4 || v.comp < 0 || v.comp > 5 || v.i < 0 || v.i > d.nx ||
        v.j < 0 || v.j > d.ny || v.k < 0 || v.k > d.nz)
      return fail(ctx, GBF_EINVAL, "gbf_upload_sources: source %d out of range", s);
    if ((v.kind == GBF_SRC_MAGNETIC) != (v.comp >= 3))
      return fail(ctx, GBF_EINVAL, "gbf_upload_sources: source %d kind/component mismatch", s);
    if (v.kind == GBF_SRC_MAGNETIC) inH.push_back(v);
    else if (v.i < d.nx && v.j < d.ny && v.k < d.nz) inE.push_back(v);
    else outE.push_back(v);
  }
  if (ntl_seen != d.ntl)
    return fail(ctx, GBF_EINVAL, "gbf_upload_sources: %d transmission lines, desc.ntl is %d", ntl_seen, d.ntl);
  std::vector<Src> all;
  all.insert(all.end(), inE.begin(), inE.end());
  all.insert(all.end(), inH.begin(), inH.end());
  all.insert(all.end(), outE.begin(), outE.end());
  CK(cudaMemcpyAsync(ctx->srcs, all.data(), sizeof(Src) * all.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->waves, waves, sizeof(float) * (size_t)d.nsrc * d.iterations,
                     cudaMemcpyHostToDevice, ctx->stream));
  invalidate_graph(ctx);
  for (int q = 0; q < kSrcInline; ++q) ctx->sp.srcqE[q] = ctx->sp.srcqH[q] = -1;
  for (size_t q = 0; q < inE.size() && q < (size_t)kSrcInline; ++q)
    ctx->sp.srcqE[q] = inE[q].i * ctx->sp.sx + inE[q].j * ctx->sp.sy + inE[q].k;
  for (size_t q = 0; q < inH.size() && q < (size_t)kSrcInline; ++q)
    ctx->sp.srcqH[q] = inH[q].i * ctx->sp.sx + inH[q].j * ctx->sp.sy + inH[q].k;
  ctx->sp.nsrcE = (int)inE.size();
  ctx->sp.srcE = ctx->srcs;
  ctx->sp.nsrcH = (int)inH.size();
  ctx->sp.srcH = ctx->srcs + inE.size();
  ctx->rp.nsrcOut = (int)outE.size();
  ctx->rp.srcOut = ctx->srcs + inE.size() + inH.size();
  return GBF_OK;
}

int gbf_set_receivers(gbf_ctx* ctx, const int32_t* coords) {
  if (!ctx) return GBF_EINVAL;
  const gbf_grid_desc& d = ctx->d;
  if (d.nrx == 0) return GBF_OK;
  if (!coords) return fail(ctx, GBF_EINVAL, "gbf_set_receivers: NULL coords");
  for (int n = 0; n < d.nrx; ++n) {
    const int x = coords[3 * n], y = coords[3 * n + 1], z = coords[3 * n + 2];
    if (x < 0 || x > d.nx || y < 0 || y > d.ny || z < 0 || z > d.nz)
      return fail(ctx, GBF_EINVAL, "gbf_set_receivers: receiver %d at (%d,%d,%d) outside the grid", n, x, y, z);
  }
  CK(cudaMemcpyAsync(ctx->rx_coords, coords, sizeof(int) * 3 * d.nrx, cudaMemcpyHostToDevice, ctx->stream));
  return GBF_OK;
}

int gbf_set_snapshots(gbf_ctx* ctx, const int32_t* defs) {
  if (!ctx) return GBF_EINVAL;
  const gbf_grid_desc& d = ctx->d;
  if (d.nsnap == 0) return GBF_OK;
  if (!defs) return fail(ctx, GBF_EINVAL, "gbf_set_snapshots: NULL defs");
  for (float* p : ctx->snaps) if (p) cudaFree(p);
  ctx->snaps.assign(d.nsnap, nullptr);
  ctx->snapdef.assign(defs, defs + 10 * d.nsnap);
  for (int s = 0; s < d.nsnap; ++s) {
    const int32_t* q = defs + 10 * s;
    const int xs = q[0], ys = q[1], zs = q[2], sdx = q[3], sdy = q[4], sdz = q[5];
    const int snx = q[6], sny = q[7], snz = q[8], time = q[9];
    if (sdx < 1 || sdy < 1 || sdz < 1 || snx < 1 || sny < 1 || snz < 1 ||
        xs < 0 || ys < 0 || zs < 0 || xs + snx * sdx > d.nx || ys + sny * sdy > d.ny ||
        zs + snz * sdz > d.nz || time < 1 || time > d.iterations)
      return fail(ctx, GBF_EINVAL, "gbf_set_snapshots: snapshot %d out of range", s);
    int rc = dev_alloc(ctx, (void**)&ctx->snaps[s], sizeof(float) * 6 * (size_t)snx * sny * snz);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return GBF_OK;
}

int gbf_reset(gbf_ctx* ctx) {
  if (!ctx) return GBF_EINVAL;
  const gbf_grid_desc& d = ctx->d;
  // a context that has not stepped, nor had fields uploaded, still holds the zeros it was
  // created with (every allocation is cleared then)
  if (ctx->dirty) {
    CK(cudaMemsetAsync(ctx->fields, 0, sizeof(float) * (ctx->fused_ok ? 12 : 6) * ctx->ncomp, ctx->stream));
    if (ctx->T) CK(cudaMemsetAsync(ctx->T, 0, sizeof(float2) * 3 * (size_t)d.maxpoles * ctx->ncomp, ctx->stream));
    if (ctx->phi_floats) CK(cudaMemsetAsync(ctx->pml_mem, 0, sizeof(float) * ctx->phi_floats, ctx->stream));
    CK(cudaMemsetAsync(ctx->rxs, 0, sizeof(float) * 9 * (size_t)d.iterations * (d.nrx + 1), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_it, 0, sizeof(int), ctx->stream));
    ctx->dirty = false;
  }
  set_current(ctx, 0);
  if (d.ntl && (int)ctx->tls_init.size() == d.ntl) {
    // line state after the incident-wave run; samples 0 of Vtotal/Itotal are that state
    CK(cudaMemcpyAsync(ctx->tls, ctx->tls_init.data(), sizeof(TLine) * d.ntl,
                       cudaMemcpyHostToDevice, ctx->stream));
    std::vector<float> out(2 * (size_t)d.ntl * d.iterations, 0.f);
    for (int n = 0; n < d.ntl; ++n) {
      const TLine& t = ctx->tls_init[n];
      out[(size_t)(2 * n) * d.iterations] = t.v[t.antpos];
      out[(size_t)(2 * n + 1) * d.iterations] = t.c[t.antpos];
    }
    CK(cudaMemcpyAsync(ctx->tl_out, out.data(), sizeof(float) * out.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->it = 0;
  return GBF_OK;
}

int gbf_upload_tls(gbf_ctx* ctx, const int32_t* info, const double* coef, const float* state,
                   const float* cell, const float* waves) {
  if (!ctx) return GBF_EINVAL;
  const gbf_grid_desc& d = ctx->d;
  if (d.ntl == 0) return GBF_OK;
  if (!info || !coef || !state || !cell || !waves)
    return fail(ctx, GBF_EINVAL, "gbf_upload_tls: NULL array");
  std::vector<TLine> tl(d.ntl);
  for (int n = 0; n < d.ntl; ++n) {
    const int32_t* q = info + 9 * n;
    TLine& t = tl[n];
    memset(&t, 0, sizeof(TLine));
    t.comp = q[0]; t.i = q[1]; t.j = q[2]; t.k = q[3]; t.first = q[4]; t.last = q[5];
    t.nl = q[6]; t.srcpos = q[7]; t.antpos = q[8];
    if (t.comp < 0 || t.comp > 2 || t.i < 0 || t.i > d.nx || t.j < 0 || t.j > d.ny || t.k < 0 ||
        t.k > d.nz || t.nl < 2 || t.nl > kTLCells || t.srcpos < 1 || t.srcpos >= t.nl ||
        t.antpos < 0 || t.antpos >= t.nl)
      return fail(ctx, GBF_EINVAL, "gbf_upload_tls: line %d out of range (at most %d cells)", n, kTLCells);
    t.s_iv = coef[4 * n]; t.s_vi = coef[4 * n + 1]; t.r = coef[4 * n + 2]; t.h = coef[4 * n + 3];
    const float* st = state + (size_t)n * (2 * kTLCells + 2);
    for (int m = 0; m < kTLCells; ++m) {
      t.v[m] = st[m];
      t.c[m] = st[kTLCells + m];
    }
    t.abcv0 = st[2 * kTLCells];
    t.abcv1 = st[2 * kTLCells + 1];
    t.d = cell[n];
    t.whole = ctx->tl_waves + (size_t)(2 * n) * d.iterations;
    t.half = ctx->tl_waves + (size_t)(2 * n + 1) * d.iterations;
  }
  CK(cudaMemcpyAsync(ctx->tl_waves, waves, sizeof(float) * 2 * (size_t)d.ntl * d.iterations,
                     cudaMemcpyHostToDevice, ctx->stream));
  ctx->tls_init = tl;
  ctx->rp.ntl = d.ntl;
  invalidate_graph(ctx);
  return gbf_reset(ctx);
}

int gbf_download_tls(gbf_ctx* ctx, float* out) {
  if (!ctx || !out) return GBF_EINVAL;
  const size_t n = 2 * (size_t)ctx->d.ntl * ctx->d.iterations;
  if (n) CK(cudaMemcpyAsync(out, ctx->tl_out, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GBF_OK;
}

}  // extern "C"

// ---- launch helpers ------------------------------------------------------------------
typedef HKernFn HKern;
typedef EKernFn EKern;

static void pick_kernels(gbf_ctx* ctx, HKern* h, EKern* e) {
  const int np = ctx->d.maxpoles, idp = ctx->idp, uh = ctx->uniform_h, tr = ctx->treal;
  switch (pml_kind(ctx->d)) {
    case PML_HORI1: kernels_pk1(np, idp, uh, tr, h, e); break;
    case PML_HORI2: kernels_pk2(np, idp, uh, tr, h, e); break;
    case PML_MRI1: kernels_pk3(np, idp, uh, tr, h, e); break;
    case PML_MRI2: kernels_pk4(np, idp, uh, tr, h, e); break;
    default: kernels_pk0(np, idp, uh, tr, h, e); break;
  }
}

// Persistent grid: as many blocks as fit on the device at once (at least one per SM).
static int persistent_blocks(const void* kern, size_t smem) {
  int dev = 0, sms = 1, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kThreads, smem);
  return sms * (per > 0 ? per : 1);
}

// The step's kernels of one context, on its stream or on `st` (a batch's).
static void launch_h(gbf_ctx* ctx, cudaStream_t st = nullptr) {
  const StepParams& p = ctx->sp;
  if (!st) st = ctx->stream;
  if (ctx->staged_h) {
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    ctx->skh<<<sms, kStagedThreads, ctx->smem_sth, st>>>(p, ctx->sgh);
    return;
  }
  HKern kern;
  EKern ek;
  pick_kernels(ctx, &kern, &ek);
  if (!ctx->grid_h) ctx->grid_h = persistent_blocks((const void*)kern, ctx->smem_h);
  dim3 block(kThreads);
  dim3 grid(ctx->grid_h);
  kern<<<grid, block, ctx->smem_h, st>>>(p);
}

// The division constants of FastDiv for divisor d >= 2 (staged.cuh).
static FastDiv fast_div(int d) {
  int l = 0;
  while ((1LL << l) < d) ++l;
  FastDiv f;
  f.m = (uint32_t)(((1ULL << (31 + l)) + (uint64_t)d - 1) / (uint64_t)d);
  f.sh = l - 1;
  return f;
}

// Geometry of a staged sweep (ELECTRIC: E, else H) with `nstream` streams per chunk behind
// `tables` bytes of coefficient tables, and the kernel's shared-memory limit; false when no ring
// of two stages fits.
static bool staged_geom(gbf_ctx* ctx, bool electric, int nstream, size_t tables, SKernFn k,
                        StagedGeom& g, size_t& smem) {
  const StepParams& p = ctx->sp;
  const gbf_grid_desc& d = ctx->d;
  const int L = kStageL, W = kStageSpan;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  g.nstream = nstream;
  // the PML profile rows of the kernel's field type after the tables, then the ring
  g.rows_off = (int)((tables + 15) & ~(size_t)15);
  int rows = 0;
  for (int s = 0; s < 6; ++s) {
    g.roff[s] = rows;
    rows += 4 * d.pml_order * d.pml_thickness[s];
  }
  g.ring_off = (int)((g.rows_off + sizeof(float) * rows + 127) & ~(size_t)127);
  g.zspan = ctx->zspan;
  g.zslots = ctx->zspan ? 4 * d.pml_order : 0;
  g.stage_floats = W * nstream + g.zslots * g.zspan;
  const size_t stage = sizeof(float) * (size_t)g.stage_floats;
  // room for the kernel's static shared memory (barriers, headers, the abort flag)
  const size_t fixed = 1024;
  int ns = kStageMax;
  while (ns >= 2 && g.ring_off + ns * stage + fixed > (size_t)optin) --ns;
  if (ns < 2) return false;
  g.nstages = ns;
  const long long plen = electric ? (long long)p.ny * p.sy : p.sx;
  const int planes = electric ? p.nx : p.nx + 1;
  g.cpp = (int)((plen + 3 + L - 1) / L);
  if ((long long)g.cpp * planes > (1LL << 31) - 1) return false;
  g.nchunks = g.cpp * planes;
  const Box& core = electric ? p.boxE[0] : p.boxH[0];
  g.ilo = core.i0;
  g.ihi = core.i0 + (core.count ? core.bi : 0);
  g.jlo = core.j0;
  g.jhi = core.j0 + (core.count ? core.bj : 0);
  g.amax = (int)(ctx->ncomp - W);   // a multiple of 4: ncomp is one of 64, W one of 8
  g.by_sy = fast_div(p.sy);
  g.by_cpp = fast_div(g.cpp < 2 ? 2 : g.cpp);
  g.err = ctx->d_err;
  g.limit_ns = 2000000000LL;
  smem = g.ring_off + ns * stage;
  return allow_dynamic_smem((const void*)k, smem, ctx->device);
}

// The staged half-steps (staged.cuh) where they apply: 3D grids with packed IDs and coefficient
// tables in shared memory whose arrays span at least two chunks; for E at most two poles (their
// state real or complex); a ring of at least two stages that fits in shared memory beside the
// tables.
// Option bit 4 keeps the plain kernels.
static void configure_staged(gbf_ctx* ctx) {
  ctx->staged = ctx->staged_h = ctx->staged_av = 0;
  ctx->sk = ctx->skh = nullptr;
  form_release(ctx);
  ctx->forms_tuned = 1;
  const gbf_grid_desc& d = ctx->d;
  const StepParams& p = ctx->sp;
  const int np = d.maxpoles;
  if ((d.options & 16) || p.two_d || ctx->idp != 1 || !p.smem) return;
  if (ctx->ncomp < 2 * (long long)kStageSpan || p.sy < 2 || p.sx < 2) return;
  SKernFn ke = nullptr, kh = nullptr;
  const int idp_h = ctx->uniform_h ? 0 : 1;
  switch (pml_kind(d)) {
    case PML_HORI1: staged_pk1(np, ctx->treal, idp_h, &ke, &kh); break;
    case PML_HORI2: staged_pk2(np, ctx->treal, idp_h, &ke, &kh); break;
    case PML_MRI1: staged_pk3(np, ctx->treal, idp_h, &ke, &kh); break;
    case PML_MRI2: staged_pk4(np, ctx->treal, idp_h, &ke, &kh); break;
    default: staged_pk0(np, ctx->treal, idp_h, &ke, &kh); break;
  }
  if (ke && np <= 2 &&
      staged_geom(ctx, true, 11 + (ctx->treal ? 3 : 6) * np, ctx->smem_e, ke, ctx->sg,
                  ctx->smem_st)) {
    ctx->sk = ke;
    ctx->staged = 1;
  }
  if (kh && staged_geom(ctx, false, 10 + idp_h, ctx->smem_h, kh, ctx->sgh, ctx->smem_sth)) {
    ctx->skh = kh;
    ctx->staged_h = 1;
  }
  ctx->staged_av = ctx->staged | (ctx->staged_h << 1);
  // staged where available until the form tuner (or an earlier model of this shape) decides
  ctx->forms_tuned = ctx->staged_av == 0 || form_cached(ctx);
}

// A staged sweep that gave up waiting for a stage leaves the error word set (read and cleared
// here, after the context's work so far has finished).
static int staged_status(gbf_ctx* ctx) {
  if (!ctx->d_err) return GBF_OK;
  int v = 0;
  CK(cudaMemcpyAsync(&v, ctx->d_err, sizeof v, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (v) {
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return fail(ctx, GBF_ECUDA, "staged half-step: a shared-memory stage was not filled within "
                "the wait limit; the fields of this run are not valid");
  }
  return GBF_OK;
}

static void launch_e(gbf_ctx* ctx, cudaStream_t st = nullptr) {
  const StepParams& p = ctx->sp;
  if (!st) st = ctx->stream;
  if (ctx->staged) {
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    ctx->sk<<<sms, kStagedThreads, ctx->smem_st, st>>>(p, ctx->sg);
    return;
  }
  HKern hk;
  EKern kern;
  pick_kernels(ctx, &hk, &kern);
  if (!ctx->grid_e) ctx->grid_e = persistent_blocks((const void*)kern, ctx->smem_e);
  dim3 block(kThreads);
  dim3 grid(ctx->grid_e);
  kern<<<grid, block, ctx->smem_e, st>>>(p);
}

static void launch_end(gbf_ctx* ctx) {
  end_of_step<<<1, 256, 0, ctx->stream>>>(ctx->sp, ctx->rp, ctx->d_it);
}

static void launch_tl(gbf_ctx* ctx) {
  if (ctx->rp.ntl)
    tl_step<<<(ctx->rp.ntl + 31) / 32, 32, 0, ctx->stream>>>(ctx->sp, ctx->tls, ctx->rp.ntl,
                                                           ctx->d.dx, ctx->d.dy, ctx->d.dz);
}

// The fused step kernel from the current buffers into the other ones; the other buffers then
// hold the current iteration. Returns the E arrays the step read.
struct EPtrs {
  const float* e[3];
};
static EPtrs launch_fused_kernel(gbf_ctx* ctx) {
  const StepParams q = fused_params(ctx);
  ctx->fk<<<ctx->f_blocks, (ctx->f_tj + 1) * 32, ctx->smem_f, ctx->stream>>>(q, ctx->ft);
  EPtrs prev;
  for (int c = 0; c < 3; ++c) prev.e[c] = q.E[c];
  set_current(ctx, ctx->cur ^ 1);
  return prev;
}

static void launch_fused_end(gbf_ctx* ctx, const EPtrs& prev) {
  RxParams r = ctx->rp;
  for (int c = 0; c < 3; ++c) r.Eold[c] = prev.e[c];
  end_of_step<<<1, 256, 0, ctx->stream>>>(ctx->sp, r, ctx->d_it);
}

static void launch_step(gbf_ctx* ctx) {
  if (ctx->fused) {
    const EPtrs prev = launch_fused_kernel(ctx);
    launch_fused_end(ctx, prev);
    return;
  }
  launch_h(ctx);
  launch_tl(ctx);
  launch_e(ctx);
  launch_end(ctx);
}

static int launch_snapshot(gbf_ctx* ctx, int s) {
  const int* q = &ctx->snapdef[10 * s];
  SnapParams sp;
  sp.xs = q[0]; sp.ys = q[1]; sp.zs = q[2]; sp.sdx = q[3]; sp.sdy = q[4]; sp.sdz = q[5];
  sp.snx = q[6]; sp.sny = q[7]; sp.snz = q[8];
  sp.out = ctx->snaps[s];
  long long n = (long long)sp.snx * sp.sny * sp.snz;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  snapshot_store<<<blocks, 256, 0, ctx->stream>>>(ctx->sp, sp);
  CK(cudaGetLastError());
  return GBF_OK;
}

static const int kGraphSteps = 16;

// ---- step tuner ------------------------------------------------------------------------
// The candidates are the fused step with each tiling and the two half-step kernels. Every one
// gives the same result bit for bit (a node's arithmetic depends on neither), so the tuner times
// real steps: the first steps of a model's run go through the candidates in turn (kTuneReps
// rounds), the step's update kernels between two events, and once all have run the fastest is
// kept (the smallest time over the rounds; the first round also carries the first-launch cost).
// The model advances as usual meanwhile. The choice is kept per model shape for the process.
// GBF_FUSED_TILE="tj,nch" forces a fused tiling; GBF_FUSED_TUNE=0 keeps the default (the fused
// step with as many chunks as give one wave of resident blocks, tile height 7).
static const int kTuneReps = 2;
struct TuneKey {
  int v[9];
  bool operator<(const TuneKey& o) const { return memcmp(v, o.v, sizeof v) < 0; }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, std::pair<int, int>> g_tune;

static TuneKey tune_key(const gbf_ctx* ctx) {
  const gbf_grid_desc& d = ctx->d;
  return TuneKey{{d.nx, d.ny, d.nz, pml_kind(d), d.maxpoles, ctx->uniform_h, ctx->treal,
                  (int)ctx->smem_f, ctx->device}};
}

static void tune_release(gbf_ctx* ctx) {
  for (cudaEvent_t e : ctx->tune_ev)
    if (e) cudaEventDestroy(e);
  ctx->tune_ev.clear();
  ctx->tune_cand.clear();
  ctx->tune_next = 0;
}

// ---- half-step form tuner ---------------------------------------------------------------
// Where a staged sweep applies, each half-step can run staged or plain, with the same results
// bit for bit; which is faster depends on the model (how much its nodes wait on memory against
// the staging's own work per chunk). The first steps of the first run of each model shape run
// two candidates in turn, every available staged sweep and the plain kernels (kTuneReps rounds),
// with three events per step that time the H half-step (with the transmission lines) and the E
// half-step apart; each half-step keeps its faster form, for the model and, per shape, for the
// process.
static std::map<TuneKey, int> g_form;

static void form_release(gbf_ctx* ctx) {
  for (cudaEvent_t e : ctx->form_ev)
    if (e) cudaEventDestroy(e);
  ctx->form_ev.clear();
  ctx->form_cand.clear();
  ctx->form_next = 0;
}

static void set_forms(gbf_ctx* ctx, int f) {
  ctx->staged = f & 1;
  ctx->staged_h = (f >> 1) & 1;
}

static bool form_cached(gbf_ctx* ctx) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto f = g_form.find(tune_key(ctx));
  if (f == g_form.end()) return false;
  set_forms(ctx, f->second & ctx->staged_av);
  return true;
}

// One timed step with the next combination; after the last one, pick.
static int form_step(gbf_ctx* ctx) {
  if (ctx->form_cand.empty()) {
    ctx->form_cand = {ctx->staged_av, 0};
    ctx->form_ev.assign(3 * ctx->form_cand.size() * kTuneReps, nullptr);
    for (auto& e : ctx->form_ev)
      if (cudaEventCreate(&e) != cudaSuccess) {
        (void)cudaGetLastError();
        form_release(ctx);
        set_forms(ctx, ctx->staged_av);
        ctx->forms_tuned = 1;
        return GBF_OK;
      }
    ctx->form_next = 0;
    invalidate_graph(ctx);
  }
  const int nc = (int)ctx->form_cand.size();
  const int q = ctx->form_next;
  set_forms(ctx, ctx->form_cand[q % nc]);
  CK(cudaEventRecord(ctx->form_ev[3 * q], ctx->stream));
  launch_h(ctx);
  launch_tl(ctx);
  CK(cudaEventRecord(ctx->form_ev[3 * q + 1], ctx->stream));
  launch_e(ctx);
  CK(cudaEventRecord(ctx->form_ev[3 * q + 2], ctx->stream));
  launch_end(ctx);
  CK(cudaGetLastError());
  ctx->form_next = q + 1;
  if (ctx->form_next < nc * kTuneReps) return GBF_OK;
  CK(cudaEventSynchronize(ctx->form_ev.back()));
  // the smallest time of each half-step in each candidate over the rounds
  std::vector<float> bh(nc, 1e30f), be(nc, 1e30f);
  for (int r = 0; r < nc * kTuneReps; ++r) {
    float mh = 0, me = 0;
    CK(cudaEventElapsedTime(&mh, ctx->form_ev[3 * r], ctx->form_ev[3 * r + 1]));
    CK(cudaEventElapsedTime(&me, ctx->form_ev[3 * r + 1], ctx->form_ev[3 * r + 2]));
    bh[r % nc] = mh < bh[r % nc] ? mh : bh[r % nc];
    be[r % nc] = me < be[r % nc] ? me : be[r % nc];
  }
  // candidate 0 holds every available staged sweep, candidate 1 none
  int pick = 0;
  if ((ctx->staged_av & 1) && be[0] < be[1]) pick |= 1;
  if ((ctx->staged_av & 2) && bh[0] < bh[1]) pick |= 2;
  set_forms(ctx, pick);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_form[tune_key(ctx)] = pick;
  }
  form_release(ctx);
  ctx->forms_tuned = 1;
  return GBF_OK;
}

// Decide whether the model needs tuning steps and set up the candidates (once).
static int tune_begin(gbf_ctx* ctx) {
  if (ctx->tuned || !ctx->tune_cand.empty()) return GBF_OK;
  invalidate_graph(ctx);
  const char* force = getenv("GBF_FUSED_TILE");
  int ftj = 0, fnch = 0;
  if (force && sscanf(force, "%d,%d", &ftj, &fnch) == 2 && configure_fused(ctx, ftj, fnch)) {
    ctx->fused = 1;
    ctx->tuned = 1;
    return GBF_OK;
  }
  const char* tune = getenv("GBF_FUSED_TUNE");
  if (tune && tune[0] == '0') {
    configure_fused(ctx, 7, 0);
    ctx->fused = 1;
    ctx->tuned = 1;
    return GBF_OK;
  }
  const TuneKey key = tune_key(ctx);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto f = g_tune.find(key);
    if (f != g_tune.end()) {
      const bool use = f->second.first && configure_fused(ctx, f->second.first, f->second.second);
      ctx->fused = use ? 1 : 0;
      ctx->tuned = 1;
      return GBF_OK;
    }
  }
  std::vector<std::pair<int, int>> cand;
  for (int tj : {7, 15}) {
    if (!configure_fused(ctx, tj, 0)) continue;
    const int base = ctx->ft.nch;
    for (int nch : {base, 2 * base, 4 * base}) {
      if (!configure_fused(ctx, tj, nch)) continue;
      const std::pair<int, int> c(tj, ctx->ft.nch);
      bool seen = false;
      for (auto& x : cand) seen |= x == c;
      if (!seen) cand.push_back(c);
    }
  }
  cand.emplace_back(0, 0);   // the two half-step kernels
  ctx->tune_ev.assign(2 * cand.size() * kTuneReps, nullptr);
  for (auto& e : ctx->tune_ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      (void)cudaGetLastError();
      tune_release(ctx);
      configure_fused(ctx, 7, 0);
      ctx->tuned = 1;
      return GBF_OK;
    }
  }
  ctx->tune_cand = cand;
  ctx->tune_next = 0;
  return GBF_OK;
}

// One step of the run with the next candidate tiling, timed; after the last one, pick.
static int tune_step(gbf_ctx* ctx) {
  const int nc = (int)ctx->tune_cand.size();
  const int q = ctx->tune_next;
  const std::pair<int, int> c = ctx->tune_cand[q % nc];
  if (c.first) {
    configure_fused(ctx, c.first, c.second);
    ctx->fused = 1;
    CK(cudaEventRecord(ctx->tune_ev[2 * q], ctx->stream));
    const EPtrs prev = launch_fused_kernel(ctx);
    CK(cudaEventRecord(ctx->tune_ev[2 * q + 1], ctx->stream));
    launch_fused_end(ctx, prev);
  } else {
    ctx->fused = 0;
    CK(cudaEventRecord(ctx->tune_ev[2 * q], ctx->stream));
    launch_h(ctx);
    launch_tl(ctx);
    launch_e(ctx);
    CK(cudaEventRecord(ctx->tune_ev[2 * q + 1], ctx->stream));
    launch_end(ctx);
  }
  CK(cudaGetLastError());
  ctx->tune_next = q + 1;
  if (ctx->tune_next < nc * kTuneReps) return GBF_OK;
  CK(cudaEventSynchronize(ctx->tune_ev.back()));
  std::vector<float> best(nc, 1e30f);
  for (int r = 0; r < nc * kTuneReps; ++r) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->tune_ev[2 * r], ctx->tune_ev[2 * r + 1]));
    if (ms < best[r % nc]) best[r % nc] = ms;
  }
  int pick = 0;
  for (int k = 1; k < nc; ++k)
    if (best[k] < best[pick]) pick = k;
  const std::pair<int, int> win = ctx->tune_cand[pick];
  if (win.first) configure_fused(ctx, win.first, win.second);
  ctx->fused = win.first ? 1 : 0;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[tune_key(ctx)] = win;
  }
  tune_release(ctx);
  ctx->tuned = 1;
  return GBF_OK;
}

static int ensure_graph(gbf_ctx* ctx) {
  if (ctx->gexec) return GBF_OK;
  // an even number of steps: a fused graph ends on the buffer it started from
  static_assert(kGraphSteps % 2 == 0, "graph steps");
  ctx->graph_cur = ctx->cur;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < kGraphSteps; ++s) launch_step(ctx);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (e != cudaSuccess) return fail(ctx, GBF_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
  ctx->graph = g;
  CK(cudaGraphInstantiate(&ctx->gexec, g, 0));
  ctx->graph_steps = kGraphSteps;
  return GBF_OK;
}

extern "C" {

int gbf_run(gbf_ctx* ctx, int nsteps, uint32_t flags) {
  if (!ctx) return GBF_EINVAL;
  if (!ctx->materials) return fail(ctx, GBF_ESTATE, "gbf_run: materials not uploaded");
  if (nsteps < 0 || ctx->it + nsteps > ctx->d.iterations)
    return fail(ctx, GBF_EINVAL, "gbf_run: %d steps from iteration %d exceed %d iterations", nsteps, ctx->it, ctx->d.iterations);
  if (nsteps > 0) ctx->dirty = true;
  if (ctx->fused_avail && !ctx->tuned && nsteps > 0) {
    int rc = tune_begin(ctx);
    if (rc) return rc;
  }
  int done = 0;
  while (done < nsteps) {
    const int it = ctx->it;
    // snapshots due at the start of this iteration (time == it + 1)
    for (int s = 0; s < ctx->d.nsnap; ++s)
      if (ctx->snapdef[10 * s + 9] == it + 1) {
        int rc = launch_snapshot(ctx, s);
        if (rc) return rc;
      }
    // steps until the next snapshot (a graph chunk never crosses one)
    int span = nsteps - done;
    for (int s = 0; s < ctx->d.nsnap; ++s) {
      const int t = ctx->snapdef[10 * s + 9] - 1;
      if (t > it && t - it < span) span = t - it;
    }
    int n = span;
    // while the half-step forms, then the fused step's tiles are being chosen: one timed
    // candidate step at a time
    while (n > 0 && !ctx->forms_tuned) {
      int rc = form_step(ctx);
      if (rc) return rc;
      --n;
    }
    while (n > 0 && ctx->fused_avail && !ctx->tuned) {
      int rc = tune_step(ctx);
      if (rc) return rc;
      --n;
    }
    if ((flags & GBF_RUN_GRAPH) && !ctx->gexec && n >= kGraphSteps) {
      int rc = ensure_graph(ctx);
      if (rc) return rc;
    }
    if ((flags & GBF_RUN_GRAPH) && ctx->gexec) {
      // the graph starts from the buffer it was captured on: one plain step realigns
      if (n > ctx->graph_steps && ctx->cur != ctx->graph_cur) {
        launch_step(ctx);
        --n;
      }
      while (n >= ctx->graph_steps && ctx->cur == ctx->graph_cur) {
        CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
        n -= ctx->graph_steps;
      }
    }
    for (int s = 0; s < n; ++s) launch_step(ctx);
    CK(cudaGetLastError());
    ctx->it += span;
    done += span;
  }
  if (flags & GBF_RUN_CHECK) {
    CK(cudaStreamSynchronize(ctx->stream));
    return staged_status(ctx);
  }
  return GBF_OK;
}

int gbf_run_timed(gbf_ctx* ctx, int nsteps, uint32_t flags, float* ms) {
  if (!ctx || !ms) return GBF_EINVAL;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->stream));
  int rc = gbf_run(ctx, nsteps, flags & ~GBF_RUN_CHECK);
  if (rc) { cudaEventDestroy(a); cudaEventDestroy(b); return rc; }
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  CK(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return GBF_OK;
}

int gbf_current_iteration(gbf_ctx* ctx, int32_t* it) {
  if (!ctx || !it) return GBF_EINVAL;
  *it = ctx->it;
  return GBF_OK;
}

int gbf_synchronize(gbf_ctx* ctx) {
  if (!ctx) return GBF_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  return GBF_OK;
}

int gbf_download_rx(gbf_ctx* ctx, float* rxs) {
  if (!ctx || !rxs) return GBF_EINVAL;
  const size_t n = 9 * (size_t)ctx->d.iterations * ctx->d.nrx;
  if (n) CK(cudaMemcpyAsync(rxs, ctx->rxs, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return staged_status(ctx);
}

int gbf_download_fields(gbf_ctx* ctx, float* fields) {
  if (!ctx || !fields) return GBF_EINVAL;
  // device arrays [6][ncomp] -> the caller's [6][npts]
  CK(cudaMemcpy2DAsync(fields, sizeof(float) * ctx->npts, current_fields(ctx),
                       sizeof(float) * ctx->ncomp, sizeof(float) * ctx->npts, 6,
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return staged_status(ctx);
}

int gbf_upload_fields(gbf_ctx* ctx, const float* fields) {
  if (!ctx || !fields) return GBF_EINVAL;
  ctx->dirty = true;
  // both buffers of a fused model: E outside the half-step's range is read from either
  for (int b = 0; b < (ctx->fused_ok ? 2 : 1); ++b)
    CK(cudaMemcpy2DAsync(ctx->fields + (size_t)b * 6 * ctx->ncomp, sizeof(float) * ctx->ncomp,
                         fields, sizeof(float) * ctx->npts, sizeof(float) * ctx->npts, 6,
                         cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GBF_OK;
}

int gbf_download_dispersive(gbf_ctx* ctx, float* T) {
  if (!ctx || !T) return GBF_EINVAL;
  if (!ctx->T) return fail(ctx, GBF_ESTATE, "gbf_download_dispersive: model has no dispersive state");
  // device arrays [3P][ncomp] -> the caller's [3P][npts]
  const int rows = 3 * ctx->d.maxpoles;
  const size_t n = (size_t)rows * ctx->npts;
  if (!ctx->treal) {
    CK(cudaMemcpy2DAsync(T, sizeof(float2) * ctx->npts, ctx->T, sizeof(float2) * ctx->ncomp,
                         sizeof(float2) * ctx->npts, rows, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GBF_OK;
  }
  // real parts on the device: copy them into the first half, then spread them out in place
  // from the end, each with its imaginary part +0
  CK(cudaMemcpy2DAsync(T, sizeof(float) * ctx->npts, ctx->T, sizeof(float) * ctx->ncomp,
                       sizeof(float) * ctx->npts, rows, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t q = n; q-- > 0;) {
    T[2 * q] = T[q];
    T[2 * q + 1] = 0.f;
  }
  return GBF_OK;
}

int gbf_download_snapshot(gbf_ctx* ctx, int s, float* out) {
  if (!ctx || !out) return GBF_EINVAL;
  if (s < 0 || s >= ctx->d.nsnap) return fail(ctx, GBF_EINVAL, "gbf_download_snapshot: bad index %d", s);
  const int* q = &ctx->snapdef[10 * s];
  const size_t n = 6 * (size_t)q[6] * q[7] * q[8];
  CK(cudaMemcpyAsync(out, ctx->snaps[s], sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GBF_OK;
}

int gbf_profile(gbf_ctx* ctx, int nsteps, float* ms_h, float* ms_e, float* ms_total) {
  if (!ctx || !ms_h || !ms_e || !ms_total) return GBF_EINVAL;
  if (!ctx->materials) return fail(ctx, GBF_ESTATE, "gbf_profile: materials not uploaded");

  if (nsteps < 0 || ctx->it + nsteps > ctx->d.iterations)
    return fail(ctx, GBF_EINVAL, "gbf_profile: too many steps");
  if (nsteps > 0) ctx->dirty = true;
  std::vector<cudaEvent_t> ev(3 * nsteps + 1);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0], ctx->stream));
  for (int s = 0; s < nsteps; ++s) {
    if (ctx->fused) {
      // one kernel for the whole step: reported in the E column, the H column stays 0
      CK(cudaEventRecord(ev[3 * s + 1], ctx->stream));
      const EPtrs prev = launch_fused_kernel(ctx);
      CK(cudaEventRecord(ev[3 * s + 2], ctx->stream));
      launch_fused_end(ctx, prev);
      CK(cudaEventRecord(ev[3 * s + 3], ctx->stream));
      continue;
    }
    launch_h(ctx);
    launch_tl(ctx);
    CK(cudaEventRecord(ev[3 * s + 1], ctx->stream));
    launch_e(ctx);
    CK(cudaEventRecord(ev[3 * s + 2], ctx->stream));
    launch_end(ctx);
    CK(cudaEventRecord(ev[3 * s + 3], ctx->stream));
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  float th = 0, te = 0, tt = 0, t;
  for (int s = 0; s < nsteps; ++s) {
    CK(cudaEventElapsedTime(&t, ev[3 * s], ev[3 * s + 1])); th += t;
    CK(cudaEventElapsedTime(&t, ev[3 * s + 1], ev[3 * s + 2])); te += t;
  }
  if (nsteps) CK(cudaEventElapsedTime(&tt, ev[0], ev[3 * nsteps]));
  for (auto& e : ev) cudaEventDestroy(e);
  ctx->it += nsteps;
  *ms_h += th; *ms_e += te; *ms_total += tt;
  return GBF_OK;
}

int gbf_set_fused_tiles(gbf_ctx* ctx, int32_t tj, int32_t nch) {
  if (!ctx) return GBF_EINVAL;
  if (!ctx->fused_avail) return fail(ctx, GBF_ESTATE, "gbf_set_fused_tiles: the model does not take the fused step");
  if (tj != 7 && tj != 15) return fail(ctx, GBF_EINVAL, "gbf_set_fused_tiles: tile height %d (7 or 15)", tj);
  tune_release(ctx);
  if (!configure_fused(ctx, tj, nch))
    return fail(ctx, GBF_EINVAL, "gbf_set_fused_tiles: no fused kernel for tile height %d and %d chunks", tj, nch);
  ctx->fused = 1;
  ctx->tuned = 1;
  invalidate_graph(ctx);
  return GBF_OK;
}

int gbf_set_step_forms(gbf_ctx* ctx, int32_t forms) {
  if (!ctx) return GBF_EINVAL;
  if (forms < 0 || forms > 3) return fail(ctx, GBF_EINVAL, "gbf_set_step_forms: forms %d (0..3)", forms);
  if (forms & ~ctx->staged_av)
    return fail(ctx, GBF_EINVAL, "gbf_set_step_forms: a staged sweep asked for (%d) does not apply "
                "to the model (available: %d)", forms, ctx->staged_av);
  form_release(ctx);
  set_forms(ctx, forms);
  ctx->forms_tuned = 1;
  invalidate_graph(ctx);
  return GBF_OK;
}

int gbf_step_info(gbf_ctx* ctx, int32_t info[8]) {
  if (!ctx || !info) return GBF_EINVAL;
  info[0] = ctx->fused;
  info[1] = ctx->fused ? ctx->f_tj : 0;
  info[2] = ctx->fused ? ctx->ft.nch : 0;
  info[3] = ctx->fused ? ctx->ft.L : 0;
  info[4] = ctx->fused ? ctx->f_blocks : 0;
  info[5] = ctx->tuned;
  info[6] = ctx->cur;
  info[7] = ctx->fused_ok | (ctx->fused_avail << 1) | (ctx->staged << 2) | (ctx->staged_h << 3) |
            (ctx->forms_tuned << 4) | (ctx->staged_av << 5);
  return GBF_OK;
}

int gbf_device_bytes(gbf_ctx* ctx, size_t* bytes) {
  if (!ctx || !bytes) return GBF_EINVAL;
  *bytes = ctx->bytes;
  return GBF_OK;
}

int gbf_set_device(int32_t device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess)
    return fail(nullptr, GBF_ECUDA, "gbf_set_device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= n)
    return fail(nullptr, GBF_EINVAL, "gbf_set_device: device %d, %d CUDA device(s) present", device, n);
  e = cudaSetDevice(device);
  if (e != cudaSuccess)
    return fail(nullptr, GBF_ECUDA, "gbf_set_device: %s", cudaGetErrorString(e));
  return GBF_OK;
}

}  // extern "C"

// ---- batches: many models advanced by one launch per half-step ------------------------
struct gbf_batch {
  std::vector<gbf_ctx*> models;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  StepParams* d_models = nullptr;
  RxParams* d_rx = nullptr;
  int* d_rangeH = nullptr;     // [n + 1]
  int* d_rangeE = nullptr;
  BKernFn hk = nullptr, ek = nullptr;
  size_t smem_h = 0, smem_e = 0;
  int grid_h = 0, grid_e = 0;
  int it = 0;
  cudaGraphExec_t gexec = nullptr;
  int graph_steps = 0;
  int tuned = 0;               // grid sizes chosen (batch_tune)
  std::vector<gbf_ctx*> own;   // models large enough to fill the GPU alone: their own kernels
  int nbatched = 0;            // models swept by the batched kernels
};

// A model with at least this many nodes fills the GPU by itself: within a batch it steps with
// its own half-step kernels (staged where they apply), the smaller ones with the batched kernels.
static const long long kBatchOwnNodes = 1LL << 21;

static int bfail(gbf_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  else g_create_err = buf;
  return code;
}

#define BK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA,           \
                   "%s failed: %s", #call, cudaGetErrorString(e_));                       \
  } while (0)

static void batch_kernels(int pk, int np, int idp, int uh, int tr, BKernFn* h, BKernFn* e) {
  switch (pk) {
    case PML_HORI1: batch_kernels_pk1(np, idp, uh, tr, h, e); break;
    case PML_HORI2: batch_kernels_pk2(np, idp, uh, tr, h, e); break;
    case PML_MRI1: batch_kernels_pk3(np, idp, uh, tr, h, e); break;
    case PML_MRI2: batch_kernels_pk4(np, idp, uh, tr, h, e); break;
    default: batch_kernels_pk0(np, idp, uh, tr, h, e); break;
  }
}

static void batch_step(gbf_batch* b) {
  BatchParams bp;
  bp.models = b->d_models;
  bp.rangeH = b->d_rangeH;
  bp.rangeE = b->d_rangeE;
  bp.n = (int)b->models.size();
  if (b->nbatched) b->hk<<<b->grid_h, kThreads, b->smem_h, b->stream>>>(bp);
  for (gbf_ctx* c : b->own) launch_h(c, b->stream);
  if (b->nbatched) b->ek<<<b->grid_e, kThreads, b->smem_e, b->stream>>>(bp);
  for (gbf_ctx* c : b->own) launch_e(c, b->stream);
  // receivers and the iteration counter of every model, batched or not
  end_of_step_batch<<<bp.n, 256, 0, b->stream>>>(b->d_models, b->d_rx);
}

// ---- batch grid tuner ----------------------------------------------------------------------
// The batched half-steps are persistent grid-stride launches: any grid size gives the same
// results, but how many blocks share the models (each block sets up every model it reaches)
// decides the time. The first steps of a batch's first run each use one candidate, k blocks
// per SM for k = 1..4 (up to what fits), twice round, timed with events; the fastest is kept
// for the batch and, per set of model shapes, for the process.
static std::mutex g_btune_mu;
static std::map<std::vector<long long>, std::pair<int, int>> g_btune;

static std::vector<long long> batch_key(const gbf_batch* b) {
  const gbf_ctx* m0 = b->models[0];
  std::vector<long long> k = {(long long)b->models.size(), pml_kind(m0->d), m0->d.maxpoles,
                              m0->idp, m0->treal, b->device};
  for (const gbf_ctx* c : b->models) {
    k.push_back(c->d.nx);
    k.push_back(c->d.ny);
    k.push_back(c->d.nz);
  }
  return k;
}

static const int kBatchTuneReps = 2;

// Returns the steps it ran (0 when the batch needs no tuning or nsteps is too short), or a
// negative status.
static int batch_tune(gbf_batch* b, int nsteps) {
  if (b->tuned) return 0;
  if (!b->nbatched) {
    b->tuned = 1;
    return 0;
  }
  const std::vector<long long> key = batch_key(b);
  {
    std::lock_guard<std::mutex> lock(g_btune_mu);
    auto f = g_btune.find(key);
    if (f != g_btune.end()) {
      b->grid_h = f->second.first;
      b->grid_e = f->second.second;
      b->tuned = 1;
      return 0;
    }
  }
  int dev = 0, sms = 1, ph = 0, pe = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ph, (const void*)b->hk, kThreads, b->smem_h);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pe, (const void*)b->ek, kThreads, b->smem_e);
  ph = ph > 0 ? ph : 1;
  pe = pe > 0 ? pe : 1;
  std::vector<std::pair<int, int>> cand;
  for (int k = 1; k <= 4; ++k) {
    const std::pair<int, int> c(sms * (k < ph ? k : ph), sms * (k < pe ? k : pe));
    bool seen = false;
    for (auto& x : cand) seen |= x == c;
    if (!seen) cand.push_back(c);
  }
  const int nc = (int)cand.size();
  if (nc < 2) {
    b->tuned = 1;
    return 0;
  }
  if (nsteps < nc * kBatchTuneReps) return 0;   // too short a run to time them; try next time
  std::vector<cudaEvent_t> ev(2 * nc * kBatchTuneReps, nullptr);
  int rc = GBF_OK;
  for (auto& e : ev)
    if (rc == GBF_OK && cudaEventCreate(&e) != cudaSuccess) rc = GBF_ECUDA;
  BatchParams bp;
  bp.models = b->d_models;
  bp.rangeH = b->d_rangeH;
  bp.rangeE = b->d_rangeE;
  bp.n = (int)b->models.size();
  for (int r = 0; r < nc * kBatchTuneReps && rc == GBF_OK; ++r) {
    const std::pair<int, int>& c = cand[r % nc];
    // a whole step: the models with their own kernels advance too (the same in every
    // candidate's time)
    cudaEventRecord(ev[2 * r], b->stream);
    b->hk<<<c.first, kThreads, b->smem_h, b->stream>>>(bp);
    for (gbf_ctx* m : b->own) launch_h(m, b->stream);
    b->ek<<<c.second, kThreads, b->smem_e, b->stream>>>(bp);
    for (gbf_ctx* m : b->own) launch_e(m, b->stream);
    cudaEventRecord(ev[2 * r + 1], b->stream);
    end_of_step_batch<<<bp.n, 256, 0, b->stream>>>(b->d_models, b->d_rx);
    if (cudaGetLastError() != cudaSuccess) rc = GBF_ECUDA;
  }
  std::vector<float> best(nc, 1e30f);
  if (rc == GBF_OK && cudaEventSynchronize(ev.back()) != cudaSuccess) rc = GBF_ECUDA;
  for (int r = 0; r < nc * kBatchTuneReps && rc == GBF_OK; ++r) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]) != cudaSuccess) rc = GBF_ECUDA;
    if (ms < best[r % nc]) best[r % nc] = ms;
  }
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (rc != GBF_OK) return bfail(b, rc, "batch tuning: %s", cudaGetErrorString(cudaGetLastError()));
  int pick = 0;
  for (int k = 1; k < nc; ++k)
    if (best[k] < best[pick]) pick = k;
  b->grid_h = cand[pick].first;
  b->grid_e = cand[pick].second;
  b->tuned = 1;
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  std::lock_guard<std::mutex> lock(g_btune_mu);
  g_btune[key] = cand[pick];
  return nc * kBatchTuneReps;
}

// The whole requested time loop as one CUDA graph (re-captured when the length changes).
static int ensure_batch_graph(gbf_batch* b, int nsteps) {
  if (b->gexec && b->graph_steps == nsteps) return GBF_OK;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < nsteps; ++s) batch_step(b);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (e != cudaSuccess) return bfail(b, GBF_ECUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(b, GBF_ECUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e));
  b->graph_steps = nsteps;
  return GBF_OK;
}

static int check_batch_steps(gbf_batch* b, int nsteps) {
  for (gbf_ctx* c : b->models)
    if (nsteps < 0 || b->it + nsteps > c->d.iterations)
      return bfail(b, GBF_EINVAL, "gbf_batch_run: %d steps from iteration %d exceed a model's %d iterations", nsteps, b->it, c->d.iterations);
  return GBF_OK;
}

extern "C" {

int gbf_batch_create(gbf_ctx* const* models, int32_t nmodels, gbf_batch** out) {
  if (!models || nmodels < 1 || !out) return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: no models");
  *out = nullptr;
  const gbf_ctx* m0 = models[0];
  if (!m0) return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: null model 0");
  const int pk = pml_kind(m0->d);
  for (int m = 0; m < nmodels; ++m) {
    const gbf_ctx* c = models[m];
    if (!c) return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: null model %d", m);
    if (!c->materials) return bfail(nullptr, GBF_ESTATE, "gbf_batch_create: model %d has no materials", m);
    if (c->device != m0->device) return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: models on different devices");
    if (pml_kind(c->d) != pk || c->d.maxpoles != m0->d.maxpoles || c->idp != m0->idp)
      return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: model %d differs in PML kind, poles or ID layout from model 0", m);
    if (c->treal != m0->treal)
      return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: model %d stores its dispersive state %s, model 0 %s (set option bit 2 on every model)",
                   m, c->treal ? "as real parts" : "complex", m0->treal ? "as real parts" : "complex");
    if (c->d.nsnap || c->d.ntl)
      return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: model %d has snapshots or transmission lines (run it alone)", m);
    if (c->it != m0->it) return bfail(nullptr, GBF_EINVAL, "gbf_batch_create: models at different iterations");
  }
  gbf_batch* b = new gbf_batch();
  b->models.assign(models, models + nmodels);
  b->device = m0->device;
  b->it = m0->it;
  auto cleanup = [&](int rc) { gbf_batch_destroy(b); return rc; };
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { bfail(nullptr, GBF_ECUDA, "gbf_batch_create: %s", cudaGetErrorString(e)); return cleanup(GBF_ECUDA); }
  std::vector<StepParams> sp(nmodels);
  std::vector<RxParams> rp(nmodels);
  std::vector<int> rh(nmodels + 1), re(nmodels + 1);
  long long h = 0, ev = 0;
  for (int m = 0; m < nmodels; ++m) {
    gbf_ctx* c = b->models[m];
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) { bfail(nullptr, GBF_ECUDA, "gbf_batch_create: model %d stream failed", m); return cleanup(GBF_ECUDA); }
    sp[m] = c->sp;
    rp[m] = c->rp;
    rh[m] = (int)h;
    re[m] = (int)ev;
    // a large model takes no part in the batched half-steps (an empty range there)
    if (c->npts >= kBatchOwnNodes && !c->sp.two_d) {
      b->own.push_back(c);
      continue;
    }
    ++b->nbatched;
    const Box& lh = c->sp.boxH[kBoxes - 1];
    const Box& le = c->sp.boxE[kBoxes - 1];
    h += ((long long)(lh.start + lh.count) + kBatchTile - 1) / kBatchTile * kBatchTile;
    ev += ((long long)(le.start + le.count) + kBatchTile - 1) / kBatchTile * kBatchTile;
    if (h > (1LL << 31) - 1 || ev > (1LL << 31) - 1) { bfail(nullptr, GBF_EINVAL, "gbf_batch_create: more than 2^31 nodes in the batch"); return cleanup(GBF_EINVAL); }
    if (c->smem_h > b->smem_h) b->smem_h = c->smem_h;
    if (c->smem_e > b->smem_e) b->smem_e = c->smem_e;
  }
  rh[nmodels] = (int)h;
  re[nmodels] = (int)ev;
  auto alloc_copy = [&](void** dst, const void* src, size_t n) {
    cudaError_t r = cudaMalloc(dst, n);
    if (r == cudaSuccess) r = cudaMemcpy(*dst, src, n, cudaMemcpyHostToDevice);
    return r;
  };
  if ((e = alloc_copy((void**)&b->d_models, sp.data(), sizeof(StepParams) * nmodels)) != cudaSuccess ||
      (e = alloc_copy((void**)&b->d_rx, rp.data(), sizeof(RxParams) * nmodels)) != cudaSuccess ||
      (e = alloc_copy((void**)&b->d_rangeH, rh.data(), sizeof(int) * (nmodels + 1))) != cudaSuccess ||
      (e = alloc_copy((void**)&b->d_rangeE, re.data(), sizeof(int) * (nmodels + 1))) != cudaSuccess) {
    bfail(nullptr, e == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA, "gbf_batch_create: %s", cudaGetErrorString(e));
    return cleanup(GBF_ECUDA);
  }
  // the ID-free H half-step when every model has one H row
  int uh = 1;
  for (int m = 0; m < nmodels; ++m) uh = uh && b->models[m]->uniform_h;
  batch_kernels(pk, m0->d.maxpoles, m0->idp, uh, m0->treal, &b->hk, &b->ek);
  const size_t sh = b->smem_h, se = b->smem_e;
  b->grid_h = persistent_blocks((const void*)b->hk, sh);
  b->grid_e = persistent_blocks((const void*)b->ek, se);
  *out = b;
  return GBF_OK;
}

void gbf_batch_destroy(gbf_batch* b) {
  if (!b) return;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->stream) cudaStreamSynchronize(b->stream);
  cudaFree(b->d_models);
  cudaFree(b->d_rx);
  cudaFree(b->d_rangeH);
  cudaFree(b->d_rangeE);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int gbf_batch_last_error(gbf_batch* b, char* buf, size_t n) {
  if (!buf || n == 0) return GBF_EINVAL;
  snprintf(buf, n, "%s", b ? b->err.c_str() : g_create_err.c_str());
  return GBF_OK;
}

int gbf_batch_run(gbf_batch* b, int32_t nsteps, uint32_t flags) {
  if (!b) return GBF_EINVAL;
  int rc = check_batch_steps(b, nsteps);
  if (rc) return rc;
  if (nsteps == 0) return GBF_OK;
  for (gbf_ctx* c : b->models) c->dirty = true;
  // the first steps of the first run time the candidate grid sizes (real steps)
  const int tuning = batch_tune(b, nsteps);
  if (tuning < 0) return tuning;
  const int rest = nsteps - tuning;
  if (rest > 0 && (flags & GBF_RUN_GRAPH)) {
    rc = ensure_batch_graph(b, rest);
    if (rc) return rc;
    BK(cudaGraphLaunch(b->gexec, b->stream));
  } else {
    for (int s = 0; s < rest; ++s) batch_step(b);
  }
  BK(cudaGetLastError());
  b->it += nsteps;
  for (gbf_ctx* c : b->models) c->it += nsteps;
  return GBF_OK;
}

int gbf_batch_run_timed(gbf_batch* b, int32_t nsteps, uint32_t flags, float* ms) {
  if (!b || !ms) return GBF_EINVAL;
  int rc0 = check_batch_steps(b, nsteps);
  if (rc0) return rc0;
  if ((flags & GBF_RUN_GRAPH) && nsteps > 0 && b->tuned) {   // capture before the timed region
    rc0 = ensure_batch_graph(b, nsteps);
    if (rc0) return rc0;
  }
  cudaEvent_t a, z;
  BK(cudaEventCreate(&a));
  BK(cudaEventCreate(&z));
  BK(cudaEventRecord(a, b->stream));
  int rc = gbf_batch_run(b, nsteps, flags);
  if (rc) { cudaEventDestroy(a); cudaEventDestroy(z); return rc; }
  BK(cudaEventRecord(z, b->stream));
  BK(cudaEventSynchronize(z));
  BK(cudaEventElapsedTime(ms, a, z));
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  return GBF_OK;
}

int gbf_batch_info(gbf_batch* b, int32_t info[4]) {
  if (!b || !info) return GBF_EINVAL;
  info[0] = b->tuned;
  info[1] = b->grid_h;
  info[2] = b->grid_e;
  info[3] = (int32_t)b->own.size();
  return GBF_OK;
}

int gbf_batch_synchronize(gbf_batch* b) {
  if (!b) return GBF_EINVAL;
  BK(cudaStreamSynchronize(b->stream));
  return GBF_OK;
}

}  // extern "C"
