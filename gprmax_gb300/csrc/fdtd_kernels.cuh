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
// Thread mapping: a persistent grid sweeps the nodes box by box (consecutive threads on
// consecutive nodes), one node per thread per pass: first the core box (whole rows away from the
// x and y slabs and faces, where only the z-slab test remains), then the x and y slab planes and
// rows, whose warps run the PML code densely. The coefficient tables are staged in shared memory
// when they fit (the reference keeps them in __constant__ memory, model_build_run.py:512-519).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbf {

constexpr int kThreads = 256;   // threads per block of the half-step kernels
// nodes a block of the batched half-steps sweeps per model visit (four per thread); each
// model's range of the batch's virtual node index is padded to a multiple of it
constexpr int kBatchTile = 4 * kThreads;
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
  float rcp;        // 1/d rounded to nearest (fp32)
  int fastdiv;      // 1: x/d may be formed from rcp (verified on the host for this d)
  int ocount;       // Phi elements per CFS order (< 2^30: a slab holds under half the nodes)
  float* phiE1;     // Phi arrays [order][...] of the first/second tangential E component
  float* phiE2;
  float* phiH1;     // H Phi read by the H update ...
  float* phiH2;
  float* phiH1n;    // ... and written (another buffer in the fused step, whose halo nodes read
  float* phiH2n;    // the H state of nodes other tiles own; the same arrays otherwise)
  const float* eR;  // [4][order][T]: RA, RB, RE, RF for E
  const float* hR;  // same for H
};

struct StepParams;
struct BatchParams;
typedef void (*HKernFn)(StepParams);
typedef void (*EKernFn)(StepParams);
typedef void (*BKernFn)(BatchParams);
// per-kind kernel tables (kernels_inst.cu, one object per PML kind)
// idp: material-ID layout (1 packed, 3 plain); uniform_h: every material has the same H row;
// treal: the dispersive state is stored as real parts (packed IDs only)
void kernels_pk0(int np, int idp, int uniform_h, int treal, HKernFn* h, EKernFn* e);
void kernels_pk1(int np, int idp, int uniform_h, int treal, HKernFn* h, EKernFn* e);
void kernels_pk2(int np, int idp, int uniform_h, int treal, HKernFn* h, EKernFn* e);
void kernels_pk3(int np, int idp, int uniform_h, int treal, HKernFn* h, EKernFn* e);
void kernels_pk4(int np, int idp, int uniform_h, int treal, HKernFn* h, EKernFn* e);
// batched forms (kernels_inst.cu)
void batch_kernels_pk0(int np, int idp, int uniform_h, int treal, BKernFn* h, BKernFn* e);
void batch_kernels_pk1(int np, int idp, int uniform_h, int treal, BKernFn* h, BKernFn* e);
void batch_kernels_pk2(int np, int idp, int uniform_h, int treal, BKernFn* h, BKernFn* e);
void batch_kernels_pk3(int np, int idp, int uniform_h, int treal, BKernFn* h, BKernFn* e);
void batch_kernels_pk4(int np, int idp, int uniform_h, int treal, BKernFn* h, BKernFn* e);

struct Src {
  int kind, comp, i, j, k, first, last, pad;
  float s0, s1;
  const float* w;   // this source's waveform table [iterations]
};

// A sweep box: nodes (i0 + a, j0 + b, k0 + c + (c >= ksplit ? kgap : 0)) for a < bi, b < bj,
// c < bk, at positions [start, start + count) of the half-step's virtual node index. Box 0 is
// the core (whole rows away from the x and y slabs and faces); boxes 1-4 are the x-minus and
// x-plus planes and the y-minus and y-plus rows between them; box 5 is spare (empty).
constexpr int kBoxes = 6;
struct Box {
  int i0, j0, k0, bi, bj, bk, ksplit, kgap;
  int start, count;
};

struct StepParams {
  float* E[3];
  float* H[3];
  float* En[3];           // fused step: where the new E and H go (the other field buffer)
  float* Hn[3];
  const uint32_t* ID[6];  // per component [ncomp]
  const uint32_t* PE;     // packed E IDs per node: x | y << 10 | z << 20 | dispersive << 30
  const uint32_t* PH;     // packed H IDs per node: x | y << 10 | z << 20
  int ncomp;              // nodes per component (< 2^31)
  int nx, ny, nz;
  int two_d;              // 1: a dimension of one cell (TMx, TMy, TMz): 2D magnetic ranges
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
  Box boxE[kBoxes];       // sweep boxes of the E half-step (domain [0,nx) x [0,ny) x [0,nz))
  Box boxH[kBoxes];       // and of the H half-step (domain [0,nx] x [0,ny] x [0,nz])
  float hrow[6];          // the H row shared by every material (DA, DBx, DBy, DBz, srcm), if any
};

// ---------------------------------------------------------------------------------------
// CFS-PML correction (pml_updates_{electric,magnetic}_{HORIPML,MRIPML}_ext.pyx).
// A node lies in at most one slab per axis (each slab is thinner than half the domain). For an
// axis, both tangential field components use the same profile row and Phi index; PmlRow holds
// that row, pml_update returns X such that the component changes by (+/-) c4 * X and advances
// the Phi recursion. RA01, IRA, RC0 ... are recomputed from the stored rows as the reference does.
struct PmlRow {
  float RA0, RB0, RE0, RF0, RA1, RB1, RE1, RF1;
};

template <int PK>
__device__ __forceinline__ PmlRow load_row(const float* __restrict__ R, int T, int pr) {
  constexpr int order = (PK == PML_HORI2 || PK == PML_MRI2) ? 2 : 1;
  PmlRow c;
  c.RA0 = __ldg(R + (0 * order + 0) * T + pr);
  c.RB0 = __ldg(R + (1 * order + 0) * T + pr);
  c.RE0 = __ldg(R + (2 * order + 0) * T + pr);
  c.RF0 = __ldg(R + (3 * order + 0) * T + pr);
  if (order == 2) {
    c.RA1 = __ldg(R + (0 * order + 1) * T + pr);
    c.RB1 = __ldg(R + (1 * order + 1) * T + pr);
    c.RE1 = __ldg(R + (2 * order + 1) * T + pr);
    c.RF1 = __ldg(R + (3 * order + 1) * T + pr);
  } else {
    c.RA1 = c.RB1 = c.RE1 = c.RF1 = 0.f;
  }
  return c;
}

// The Phi state's present values are ph0 (and ph1, the second CFS order, at pidx + ocount); its
// next value is written to `out` (the array read, except for the H state of the fused step),
// and only when `wr` (a halo node recomputed by a tile that does not own it reads the state but
// leaves it to its owner).
template <int PK>
__device__ __forceinline__ float pml_update_v(float dF, float ph0, float ph1, float* out, int pidx,
                                              int ocount, const PmlRow& c, bool wr) {
  if (PK == PML_HORI1) {
    const float RA01 = c.RA0 - 1.0f;
    const float X = RA01 * dF + c.RB0 * ph0;
    if (wr) out[pidx] = c.RE0 * ph0 - c.RF0 * dF;
    return X;
  } else if (PK == PML_HORI2) {
    const float RA01 = c.RA0 * c.RA1 - 1.0f;
    const float X = RA01 * dF + c.RA1 * c.RB0 * ph0 + c.RB1 * ph1;
    if (wr) {
      out[pidx + ocount] = c.RE1 * ph1 - c.RF1 * (c.RA0 * dF + c.RB0 * ph0);
      out[pidx] = c.RE0 * ph0 - c.RF0 * dF;
    }
    return X;
  } else if (PK == PML_MRI1) {
    const float IRA = 1.0f / c.RA0;
    const float IRA1 = IRA - 1.0f;
    const float RC0 = IRA * c.RB0 * c.RF0;
    const float X = IRA1 * dF - IRA * ph0;
    if (wr) out[pidx] = c.RE0 * ph0 + RC0 * dF - RC0 * ph0;
    return X;
  } else {  // PML_MRI2
    const float IRA = 1.0f / (c.RA0 + c.RA1);
    const float IRA1 = IRA - 1.0f;
    const float RC0 = IRA * c.RF0;
    const float RC1 = IRA * c.RF1;
    const float Psi = c.RB0 * ph0 + c.RB1 * ph1;
    const float X = IRA1 * dF - IRA * Psi;
    if (wr) {
      out[pidx + ocount] = c.RE1 * ph1 + RC1 * (dF - Psi);
      out[pidx] = c.RE0 * ph0 + RC0 * (dF - Psi);
    }
    return X;
  }
}

// The same with the state read from `in`.
template <int PK>
__device__ __forceinline__ float pml_update(float dF, const float* in, float* out, int pidx,
                                            int ocount, const PmlRow& c, bool wr) {
  constexpr bool two = PK == PML_HORI2 || PK == PML_MRI2;
  const float ph0 = in[pidx];
  const float ph1 = two ? in[pidx + ocount] : 0.f;
  return pml_update_v<PK>(dF, ph0, ph1, out, pidx, ocount, c, wr);
}

// x / d rounded to nearest, as IEEE division gives it. When the host has verified d
// (Slab::fastdiv), the quotient comes from the correctly rounded reciprocal r with one
// residual correction (Markstein, IBM J. Res. Develop. 34(1), 1990): q = x*r, e = x - q*d
// (exact, one fused multiply-add), result q + e*r. The correction is used while |x| lies in
// [2^-60, 2^80), where q, e and e*r stay normal for cell sizes in [2^-20, 2^20]; zeros keep q
// (which carries their sign) and every other x takes the division.
constexpr uint32_t kDivLo = 67u << 23;    // bits of 2^-60
constexpr uint32_t kDivHi = 207u << 23;   // bits of 2^80
__device__ __forceinline__ float div_cell(float x, float d, float r, int fast) {
  if (fast) {
    const float q = __fmul_rn(x, r);
    const uint32_t ax = __float_as_uint(x) & 0x7fffffffu;
    if (ax - kDivLo < kDivHi - kDivLo) return __fmaf_rn(__fmaf_rn(-q, d, x), r, q);
    if (ax == 0u) return q;
  }
  return __fdiv_rn(x, d);
}

// Phi index of node (i, j, k) at profile index pr (layouts: x [pr][j][k], y [i][pr][k],
// z [i][j][pr]).
template <int AXIS>
__device__ __forceinline__ int phi_index(int i, int j, int k, int pr, int T, int ny, int nz) {
  if (AXIS == 0) return (pr * ny + j) * nz + k;
  if (AXIS == 1) return (i * T + pr) * nz + k;
  return (i * ny + j) * T + pr;
}

// Slab membership of coordinate c along one axis (n cells, minus/plus thickness Tm/Tp).
// E ranges: minus c in [1, Tm] (pr = Tm - c), plus c in [n - Tp, n - 1] (pr = c - (n - Tp)).
// H ranges: minus c in [0, Tm - 1] (pr = Tm - 1 - c), plus as E.
// Returns 0 outside, 1 in the minus slab, 2 in the plus slab.
template <bool ELECTRIC>
__device__ __forceinline__ int axis_member(int c, int n, int Tm, int Tp, int& pr) {
  const int pm = ELECTRIC ? Tm - c : Tm - 1 - c;
  const int pp = c - (n - Tp);
  const bool inm = (unsigned)pm < (unsigned)Tm;
  const bool inp = (unsigned)pp < (unsigned)Tp;
  pr = inp ? pp : pm;
  return inp ? 2 : (inm ? 1 : 0);
}

// The two X values of one axis for the node: first/second tangential component (x: y, z;
// y: x, z; z: x, y) with their Phi arrays 1 and 2. `where` is axis_member's result (1 or 2).
template <int PK, bool ELECTRIC, int AX>
__device__ __forceinline__ void pml_axis(const StepParams& p, int where, int pr, int i, int j,
                                         int k, float dA, float dB, float& XA, float& XB,
                                         bool wr = true) {
  // the two slabs of the axis are selected field by field, which keeps every parameter read a
  // constant-bank operand (no indexed parameter loads)
  const Slab& m = p.slab[AX];
  const Slab& q = p.slab[AX + 3];
  const bool plus = where == 2;
  const int T = plus ? q.T : m.T;
  const int pidx = phi_index<AX>(i, j, k, pr, T, p.ny, p.nz);
  const float* R = ELECTRIC ? (plus ? q.eR : m.eR) : (plus ? q.hR : m.hR);
  const PmlRow c = load_row<PK>(R, T, pr);
  const float d = m.d, r = m.rcp;   // the same cell size on both sides of an axis
  const int fast = m.fastdiv;
  const int ocount = plus ? q.ocount : m.ocount;
  float* ph1 = ELECTRIC ? (plus ? q.phiE1 : m.phiE1) : (plus ? q.phiH1 : m.phiH1);
  float* ph2 = ELECTRIC ? (plus ? q.phiE2 : m.phiE2) : (plus ? q.phiH2 : m.phiH2);
  float* out1 = ELECTRIC ? ph1 : (plus ? q.phiH1n : m.phiH1n);
  float* out2 = ELECTRIC ? ph2 : (plus ? q.phiH2n : m.phiH2n);
  XA = pml_update<PK>(div_cell(dA, d, r, fast), ph1, out1, pidx, ocount, c, wr);
  XB = pml_update<PK>(div_cell(dB, d, r, fast), ph2, out2, pidx, ocount, c, wr);
}

// Sign with which axis AX's X enters component C: H x-axis Hy +, Hz -; y-axis Hx -, Hz +;
// z-axis Hx +, Hy -. E has the opposite signs.
template <bool ELECTRIC, int AX, int C>
__host__ __device__ static constexpr bool pml_plus() {
  return ELECTRIC != ((AX == 0) ? (C == 1) : (AX == 1) ? (C == 2) : (C == 0));
}

// Apply the slab corrections of component C (tangential axes a < b) in the reference's slab
// order x0, y0, z0, xmax, ymax, zmax: b comes first only when the node is in a's plus slab and
// in b's minus slab. Each correction is F +/- c4 * X.
template <bool ELECTRIC, int C>
__device__ __forceinline__ float apply_pml(float F, float c4, const int* where, const float* XA,
                                           const float* XB) {
  constexpr int a = C == 0 ? 1 : 0;
  constexpr int b = C == 2 ? 1 : 2;
  // C is the first tangential component of axis a when a == 0 ? C == 1 : C == 0
  const float ta = c4 * ((a == 0 ? C == 1 : C == 0) ? XA[a] : XB[a]);
  const float tb = c4 * ((b == 0 ? C == 1 : C == 0) ? XA[b] : XB[b]);
  constexpr bool pa = pml_plus<ELECTRIC, a, C>();
  constexpr bool pb = pml_plus<ELECTRIC, b, C>();
  const bool ina = where[a] != 0, inb = where[b] != 0;
  if (ina && inb && where[a] == 2 && where[b] == 1) {
    F = pb ? F + tb : F - tb;
    F = pa ? F + ta : F - ta;
  } else {
    if (ina) F = pa ? F + ta : F - ta;
    if (inb) F = pb ? F + tb : F - tb;
  }
  return F;
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
// Persistent sweep: a grid of a few blocks per SM strides through each box's nodes in order
// (consecutive threads on consecutive nodes), so every array is streamed front to back by the
// whole GPU at once; neighbours along j, k (and x) are re-reads served by L1/L2. The position in
// the box advances incrementally: the grid stride splits into whole planes, rows and nodes.
struct BoxWalk {
  int a, b, c, sa, sb, sc;
  __device__ __forceinline__ BoxWalk(int q, int stride, const Box& B) {
    const int plane = B.bj * B.bk;
    a = q / plane;
    int r = q - a * plane;
    b = r / B.bk;
    c = r - b * B.bk;
    sa = stride / plane;
    r = stride - sa * plane;
    sb = r / B.bk;
    sc = r - sb * B.bk;
  }
  __device__ __forceinline__ void advance(const Box& B) {
    c += sc;
    if (c >= B.bk) { c -= B.bk; ++b; }
    b += sb;
    if (b >= B.bj) { b -= B.bj; ++a; }
    a += sa;
  }
  __device__ __forceinline__ int k(const Box& B) const {
    return B.k0 + c + (c >= B.ksplit ? B.kgap : 0);
  }
};

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

// Coefficients of the H half-step: per-material rows (C4: DA, DBx, DBy, DBz; Cs: srcm) indexed
// by the node's material numbers, or, with IDP == 0 (every material has the same H row, as in
// any model without magnetic materials), that one row from the kernel parameters (constant
// bank, no registers held) and no material numbers loaded at all.
struct HCoef {
  const float4* C4;
  const float* Cs;
};
template <int IDP>
__device__ __forceinline__ float4 hrow(const StepParams& p, const HCoef& c, uint32_t m) {
  return IDP == 0 ? make_float4(p.hrow[0], p.hrow[1], p.hrow[2], p.hrow[3]) : c.C4[m];
}
template <int IDP>
__device__ __forceinline__ float hsrcm(const StepParams& p, const HCoef& c, uint32_t m) {
  return IDP == 0 ? p.hrow[4] : c.Cs[m];
}

// H update of one node: main update (update_magnetic), slab corrections in slab order, sources.
// where[a] / pr[a]: slab membership and profile index along each axis (axis_member; 0 outside
// the PML). The X values of the node's slabs are formed first (they depend only on the E
// differences and the Phi state), then each component takes its main update and its
// corrections in the reference's order.
// h_node_x takes the slab X values already formed (XA, XB per axis; zero off the slabs).
// THREE_D: the caller runs only for 3D grids (the 2D gating is then known to pass).
template <int PK, int IDP, bool CORE, bool THREE_D = false>
__device__ __forceinline__ void h_node_x(const StepParams& p, const HCoef& hc,
                                         int i, int j, int k, bool src, int it, const int* where,
                                         const float* XA, const float* XB, float dEz_y,
                                         float dEy_z, float dEx_z, float dEz_x, float dEy_x,
                                         float dEx_y, uint32_t mx, uint32_t my, uint32_t mz,
                                         float& hx, float& hy, float& hz) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const bool iin = CORE || i < nx, jin = CORE || j < ny, kin = k < nz;
  const bool ipos = CORE || i >= 1, jpos = CORE || j >= 1;
  // 2D grids (update_magnetic's 2D branch, fields_updates_ext.pyx:377-400): Hx only when ny or
  // nz is one cell and only below i = nx; Hy, Hz likewise along j and k
  const bool hx2 = THREE_D || !p.two_d || ((ny == 1 || nz == 1) && iin);
  const bool hy2 = THREE_D || !p.two_d || ((nx == 1 || nz == 1) && jin);
  const bool hz2 = THREE_D || !p.two_d || ((nx == 1 || ny == 1) && kin);
  // Hx: main i in [1,nx], j in [0,ny), k in [0,nz); slabs along y and z
  {
    const bool mainu = ipos && jin && kin && hx2;
    const bool pml = PK != PML_NONE && (where[1] || where[2]);
    // the main update is formed on every node and kept where it applies (no branch)
    const float4 c = hrow<IDP>(p, hc, mx);
    const float Fo = hx;
    float F = c.x * Fo - c.z * dEz_y + c.w * dEy_z;
    F = mainu ? F : Fo;
    if (pml) F = apply_pml<false, 0>(F, hsrcm<IDP>(p, hc, mx), where, XA, XB);
    if (src) F = apply_h_sources(F, 3, i, j, k, it, hsrcm<IDP>(p, hc, mx), p);
    hx = F;
  }
  // Hy: main i in [0,nx), j in [1,ny], k in [0,nz); slabs along x and z
  {
    const bool mainu = iin && jpos && kin && hy2;
    const bool pml = PK != PML_NONE && (where[0] || where[2]);
    // the main update is formed on every node and kept where it applies (no branch)
    const float4 c = hrow<IDP>(p, hc, my);
    const float Fo = hy;
    float F = c.x * Fo - c.w * dEx_z + c.y * dEz_x;
    F = mainu ? F : Fo;
    if (pml) F = apply_pml<false, 1>(F, hsrcm<IDP>(p, hc, my), where, XA, XB);
    if (src) F = apply_h_sources(F, 4, i, j, k, it, hsrcm<IDP>(p, hc, my), p);
    hy = F;
  }
  // Hz: main i in [0,nx), j in [0,ny), k in [1,nz]; slabs along x and y
  {
    const bool mainu = iin && jin && (k >= 1) && hz2;
    const bool pml = PK != PML_NONE && (where[0] || where[1]);
    // the main update is formed on every node and kept where it applies (no branch)
    const float4 c = hrow<IDP>(p, hc, mz);
    const float Fo = hz;
    float F = c.x * Fo - c.y * dEy_x + c.z * dEx_y;
    F = mainu ? F : Fo;
    if (pml) F = apply_pml<false, 2>(F, hsrcm<IDP>(p, hc, mz), where, XA, XB);
    if (src) F = apply_h_sources(F, 5, i, j, k, it, hsrcm<IDP>(p, hc, mz), p);
    hz = F;
  }
}

template <int PK, int IDP, bool CORE>
__device__ __forceinline__ void h_node(const StepParams& p, const HCoef& hc,
                                       int i, int j, int k, bool src, int it, const int* where,
                                       const int* pr, float dEz_y, float dEy_z, float dEx_z,
                                       float dEz_x, float dEy_x, float dEx_y, uint32_t mx,
                                       uint32_t my, uint32_t mz, float& hx, float& hy, float& hz,
                                       bool wphi = true) {
  float XA[3] = {0.f, 0.f, 0.f}, XB[3] = {0.f, 0.f, 0.f};
  if (PK != PML_NONE) {
    if (!CORE && where[0]) pml_axis<PK, false, 0>(p, where[0], pr[0], i, j, k, dEz_x, dEy_x, XA[0], XB[0], wphi);
    if (!CORE && where[1]) pml_axis<PK, false, 1>(p, where[1], pr[1], i, j, k, dEz_y, dEx_y, XA[1], XB[1], wphi);
    if (where[2]) pml_axis<PK, false, 2>(p, where[2], pr[2], i, j, k, dEy_z, dEx_z, XA[2], XB[2], wphi);
  }
  h_node_x<PK, IDP, CORE>(p, hc, i, j, k, src, it, where, XA, XB, dEz_y, dEy_z, dEx_z, dEz_x,
                          dEy_x, dEx_y, mx, my, mz, hx, hy, hz);
}

// One H node at (i, j, k): loads, update, stores. CORE: the node lies in the core box (i and j
// in [1, n-1] and outside the x and y slabs), so only k decides neighbours and PML terms.
template <int PK, int IDP, bool CORE>
__device__ __forceinline__ void h_site(const StepParams& p, const HCoef& hc,
                                       int i, int j, int k, int it) {
  const int nx = p.nx, ny = p.ny, nz = p.nz, sx = p.sx, sy = p.sy;
  const int idx = i * sx + j * sy + k;
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  float* __restrict__ Hx = p.H[0];
  float* __restrict__ Hy = p.H[1];
  float* __restrict__ Hz = p.H[2];
  const bool iin = CORE || i < nx, jin = CORE || j < ny, kin = k < nz;
  // issue every load of the node before any store
  const float ex_c = __ldg(Ex + idx), ey_c = __ldg(Ey + idx), ez_c = __ldg(Ez + idx);
  const float ex_j = jin ? __ldg(Ex + idx + sy) : 0.f;
  const float ez_j = jin ? __ldg(Ez + idx + sy) : 0.f;
  const float ex_k = kin ? __ldg(Ex + idx + 1) : 0.f;
  const float ey_k = kin ? __ldg(Ey + idx + 1) : 0.f;
  const float ey_n = iin ? __ldg(Ey + idx + sx) : 0.f;
  const float ez_n = iin ? __ldg(Ez + idx + sx) : 0.f;
  uint32_t mx = 0, my = 0, mz = 0;
  if (IDP == 0) {
    // one H row for every material: no material numbers needed
  } else if (IDP == 1) {
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
  int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
  if (PK != PML_NONE && iin && jin && kin) {
    if (!CORE) {
      where[0] = axis_member<false>(i, nx, p.slab[0].T, p.slab[3].T, pr[0]);
      where[1] = axis_member<false>(j, ny, p.slab[1].T, p.slab[4].T, pr[1]);
    }
    where[2] = axis_member<false>(k, nz, p.slab[2].T, p.slab[5].T, pr[2]);
  }
  const bool src = p.nsrcH && node_has_source(idx, p.nsrcH, p.srcqH, p.srcH, sx, sy);
  h_node<PK, IDP, CORE>(p, hc, i, j, k, src, it, where, pr, ez_j - ez_c, ey_k - ey_c, ex_k - ex_c,
                   ez_n - ez_c, ey_n - ey_c, ex_j - ex_c, mx, my, mz, hx, hy, hz);
  Hx[idx] = hx;
  Hy[idx] = hy;
  Hz[idx] = hz;
}

// H half-step. Domain: i in [0, nx], j in [0, ny], k in [0, nz] (every node of the arrays),
// swept box by box (core first) by one persistent grid.
// The H sweep of one model over its boxes. q is the thread's position in the launch's virtual
// node index and base the position of the model's first node there; returns q after the
// model's last node. TILE: the sweep also stops at position lim (a batch tile's end).
template <int PK, int IDP, bool TILE = false>
__device__ __forceinline__ int h_sweep(const StepParams& p, const HCoef& hc,
                                       int q, int base, int stride, int it, int lim = 0) {
  q -= base;
  lim -= base;   // TILE: positions from lim on belong to another block
  {
    const Box& B = p.boxH[0];
    const int end = B.start + B.count;
    if (q < end && (!TILE || q < lim)) {
      BoxWalk w(q - B.start, stride, B);
      for (; q < end && (!TILE || q < lim); q += stride, w.advance(B))
        h_site<PK, IDP, true>(p, hc, B.i0 + w.a, B.j0 + w.b, w.k(B), it);
    }
  }
#pragma unroll 1
  for (int b = 1; b < kBoxes; ++b) {
    if (TILE && q >= lim) break;
    const Box& B = p.boxH[b];
    const int end = B.start + B.count;
    if (q >= end) continue;
    BoxWalk w(q - B.start, stride, B);
    for (; q < end && (!TILE || q < lim); q += stride, w.advance(B))
      h_site<PK, IDP, false>(p, hc, B.i0 + w.a, B.j0 + w.b, w.k(B), it);
  }
  return q + base;
}

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
  HCoef hc;
  hc.C4 = p.smem ? s4 : p.cH4;
  hc.Cs = p.smem ? ss : p.cHs;
  int it = 0;
  if (p.nsrcH) it = *p.d_it;
  h_sweep<PK, IDP>(p, hc, blockIdx.x * blockDim.x + threadIdx.x, 0, gridDim.x * blockDim.x, it);
}

// ---------------------------------------------------------------------------------------
// Batched half-steps: many models advance in one launch. The launch's virtual node index is
// the concatenation of the models' sweeps, each padded to whole tiles of kBatchTile nodes
// (range[m] .. range[m+1]). Blocks take tiles in turn (tile t = blockIdx.x, + gridDim.x, ...);
// a tile lies in one model, so on reaching it a block copies that model's parameters (and
// coefficient tables) into shared memory and sweeps the tile's nodes, four per thread. (A grid
// stride over the whole index would give a block one node per thread of each small model it
// passes, and a set-up for each.)
struct BatchParams {
  const StepParams* models;   // [n] device copies of the models' parameters
  const int* rangeH;          // [n + 1] starts of the models' H sweeps (multiples of kBatchTile)
  const int* rangeE;          // [n + 1] same for the E sweeps
  int n;
};

__device__ __forceinline__ void load_params(StepParams& dst, const StepParams* src) {
  static_assert(sizeof(StepParams) % 8 == 0, "StepParams size");
  const unsigned long long* a = reinterpret_cast<const unsigned long long*>(src);
  unsigned long long* b = reinterpret_cast<unsigned long long*>(&dst);
  for (int w = threadIdx.x; w < (int)(sizeof(StepParams) / 8); w += blockDim.x) b[w] = a[w];
}

template <int PK, int IDP>
__global__ void __launch_bounds__(kThreads, 4)
h_half_step_batch(const __grid_constant__ BatchParams bp) {
  __shared__ StepParams p;
  extern __shared__ float4 smem_hb[];
  const int total = __ldg(bp.rangeH + bp.n);
  int m = 0, mend = -1;   // the model whose parameters are loaded (none yet) and its range end
  int mbeg = 0, it = 0;
  HCoef hc;
#pragma unroll 1
  for (int t0 = blockIdx.x * kBatchTile; t0 < total; t0 += gridDim.x * kBatchTile) {
    if (t0 >= mend) {
      // the tile's model: ranges ascend and are whole tiles (empty for models with their own
      // kernels), and t0 < total keeps m < n
      while (__ldg(bp.rangeH + m + 1) <= t0) ++m;
      mbeg = __ldg(bp.rangeH + m);
      mend = __ldg(bp.rangeH + m + 1);
      __syncthreads();
      load_params(p, bp.models + m);
      __syncthreads();
      float4* s4 = smem_hb;
      float* ss = reinterpret_cast<float*>(s4 + (p.smem ? p.nmat : 0));
      if (p.smem) stage_tables(p, false, s4, ss, nullptr);
      __syncthreads();
      hc.C4 = p.smem ? s4 : p.cH4;
      hc.Cs = p.smem ? ss : p.cHs;
      it = p.nsrcH ? *p.d_it : 0;
    }
    h_sweep<PK, IDP, true>(p, hc, t0 + threadIdx.x, mbeg, blockDim.x, it, t0 + kBatchTile);
  }
}

// ---------------------------------------------------------------------------------------
// Electric sources at one node/component, in list order (voltage sources, transmission lines,
// Hertzian dipoles; model_build_run.py:459-461): sources.py:81-120, :396-424 and :163-193 with
// numpy-2 fp32 operation order.
__device__ __forceinline__ float apply_e_sources(float F, int comp, int i, int j, int k, int it,
                                                 float c4, const StepParams& p) {
  for (int s = 0; s < p.nsrcE; ++s) {
    const Src& q = p.srcE[s];
    if (q.comp != comp || q.i != i || q.j != j || q.k != k) continue;
    if (it < q.first || it > q.last) continue;
    if (q.kind == 4) {        // transmission line: -V/d from the line (tl_step), w -> that value
      F = *q.w;
      continue;
    }
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

// E update of one node for all three components: main update (update_electric, or part A of
// the dispersive update), slab corrections in slab order, sources, dispersive part B.
// where[a] / pr[a]: slab membership and profile index along each axis (0 outside the PML).
// e_node_x takes the slab X values already formed (XA, XB per axis; zero off the slabs).
template <int PK, int NP, bool CORE, bool TR>
__device__ __forceinline__ void e_node_x(const StepParams& p, const float4* C4, const float* Cs,
                                         const float2* CD, int i, int j, int k, bool src, int it,
                                         const int* where, const float* XA, const float* XB,
                                         const uint32_t* m, float* e,
                                         float2 (*t)[NP > 0 ? NP : 1], float dHz_y, float dHy_z,
                                         float dHx_z, float dHz_x, float dHy_x, float dHx_y) {
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    bool mainu, pml;
    if (comp == 0) {
      mainu = (CORE || j >= 1) && (k >= 1);
      pml = where[1] || where[2];
    } else if (comp == 1) {
      mainu = (CORE || i >= 1) && (k >= 1);
      pml = where[0] || where[2];
    } else {
      mainu = CORE || ((i >= 1) && (j >= 1));
      pml = where[0] || where[1];
    }
    if (PK == PML_NONE) pml = false;
    const uint32_t mm = m[comp];
    const float Eold = e[comp];
    float2 TA[NP > 0 ? NP : 1];
    // the main update is formed on every node and kept where it applies (no branch); curl
    // terms in the reference's order: CA*E + CB1*d1 - CB2*d2
    const float4 c = C4[mm];
    float t1, t2;
    if (comp == 0) { t1 = c.z * dHz_y; t2 = c.w * dHy_z; }
    else if (comp == 1) { t1 = c.w * dHx_z; t2 = c.y * dHz_x; }
    else { t1 = c.y * dHy_x; t2 = c.z * dHx_y; }
    float F;
    if (NP == 0) {
      F = c.x * Eold + t1 - t2;
    } else if (TR) {
      // real pole state: per material and pole (Re(e0*eqt2), Re(eqt), Re(zt), srce). The
      // complex update's Im(eqt)*Im(T) term is (+0)*(+0) = +0 here and x - (+0) == x, so it is
      // left out; every other operation is the complex update's real part, in its order.
      float phi = 0.f;
      const float4* rec = reinterpret_cast<const float4*>(CD) + mm * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float4 r = rec[q];
        const float Tx = t[comp][q].x;
        phi = phi + r.x * Tx;
        TA[q].x = r.y * Tx + r.z * Eold;
        TA[q].y = 0.f;
      }
      F = c.x * Eold + t1 - t2 - rec[0].w * phi;
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
    F = mainu ? F : Eold;
    if (PK != PML_NONE && pml) {
      const float c4 = Cs[mm];
      if (comp == 0) F = apply_pml<true, 0>(F, c4, where, XA, XB);
      else if (comp == 1) F = apply_pml<true, 1>(F, c4, where, XA, XB);
      else F = apply_pml<true, 2>(F, c4, where, XA, XB);
    }
    if (src) F = apply_e_sources(F, comp, i, j, k, it, Cs[mm], p);
    e[comp] = F;
    if (NP > 0 && TR) {
      const float4* rec = reinterpret_cast<const float4*>(CD) + mm * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float tx = TA[q].x - rec[q].z * F;
        t[comp][q].x = mainu ? tx : t[comp][q].x;
      }
    } else if (NP > 0) {
      const float2* cd = CD + mm * 3 * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float2 z = cd[3 * q + 2];
        const float tx = TA[q].x - z.x * F, ty = TA[q].y - z.y * F;
        t[comp][q].x = mainu ? tx : t[comp][q].x;
        t[comp][q].y = mainu ? ty : t[comp][q].y;
      }
    }
  }
}

template <int PK, int NP, bool CORE, bool TR>
__device__ __forceinline__ void e_node(const StepParams& p, const float4* C4, const float* Cs,
                                       const float2* CD, int i, int j, int k, bool src, int it,
                                       const int* where, const int* pr, float dHz_y,
                                       float dHy_z, float dHx_z, float dHz_x, float dHy_x,
                                       float dHx_y, const uint32_t* m, float* e, float2 (*t)[NP > 0 ? NP : 1]) {
  float XA[3] = {0.f, 0.f, 0.f}, XB[3] = {0.f, 0.f, 0.f};
  if (PK != PML_NONE) {
    if (!CORE && where[0]) pml_axis<PK, true, 0>(p, where[0], pr[0], i, j, k, dHz_x, dHy_x, XA[0], XB[0]);
    if (!CORE && where[1]) pml_axis<PK, true, 1>(p, where[1], pr[1], i, j, k, dHz_y, dHx_y, XA[1], XB[1]);
    if (where[2]) pml_axis<PK, true, 2>(p, where[2], pr[2], i, j, k, dHy_z, dHx_z, XA[2], XB[2]);
  }
  e_node_x<PK, NP, CORE, TR>(p, C4, Cs, CD, i, j, k, src, it, where, XA, XB, m, e, t, dHz_y, dHy_z,
                             dHx_z, dHz_x, dHy_x, dHx_y);
}

// One E node at (i, j, k): loads, update, stores. CORE: the node lies in the core box (i and j
// >= 1 and outside the x and y slabs), so only k decides neighbours and PML terms.
template <int PK, int NP, int IDP, bool CORE, bool TR>
__device__ __forceinline__ void e_site(const StepParams& p, const float4* C4, const float* Cs,
                                       const float2* CD, int i, int j, int k, int it) {
  const int sx = p.sx, sy = p.sy;
  const int idx = i * sx + j * sy + k;
  const float* __restrict__ Hx = p.H[0];
  const float* __restrict__ Hy = p.H[1];
  const float* __restrict__ Hz = p.H[2];
  constexpr int NPV = NP > 0 ? NP : 1;
  // issue every load of the node before any store
  const float hx_c = __ldg(Hx + idx), hy_c = __ldg(Hy + idx), hz_c = __ldg(Hz + idx);
  const float hx_j = (CORE || j >= 1) ? __ldg(Hx + idx - sy) : 0.f;
  const float hz_j = (CORE || j >= 1) ? __ldg(Hz + idx - sy) : 0.f;
  const float hx_k = k >= 1 ? __ldg(Hx + idx - 1) : 0.f;
  const float hy_k = k >= 1 ? __ldg(Hy + idx - 1) : 0.f;
  const float hy_p = (CORE || i >= 1) ? __ldg(Hy + idx - sx) : 0.f;
  const float hz_p = (CORE || i >= 1) ? __ldg(Hz + idx - sx) : 0.f;
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
    for (int qq = 0; qq < NP; ++qq) {
      const long long o = (comp * NP + qq) * (long long)p.ncomp + idx;
      // TR: the state is stored as its real part; its imaginary part is +0 at every step
      t[comp][qq] = TR ? make_float2(reinterpret_cast<const float*>(p.T)[o], 0.f) : p.T[o];
    }
  }
  int where[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
  if (PK != PML_NONE) {
    if (!CORE) {
      where[0] = axis_member<true>(i, p.nx, p.slab[0].T, p.slab[3].T, pr[0]);
      where[1] = axis_member<true>(j, p.ny, p.slab[1].T, p.slab[4].T, pr[1]);
    }
    where[2] = axis_member<true>(k, p.nz, p.slab[2].T, p.slab[5].T, pr[2]);
  }
  const bool src = p.nsrcE && node_has_source(idx, p.nsrcE, p.srcqE, p.srcE, sx, sy);
  e_node<PK, NP, CORE, TR>(p, C4, Cs, CD, i, j, k, src, it, where, pr, hz_c - hz_j, hy_c - hy_k,
                       hx_c - hx_k, hz_c - hz_p, hy_c - hy_p, hx_c - hx_j, m, e, t);
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

// E half-step. Domain: i in [0, nx), j in [0, ny), k in [0, nz), swept box by box (core
// first) by one persistent grid. NP = dispersive poles.
// The E sweep of one model over its boxes (see h_sweep).
template <int PK, int NP, int IDP, bool TR, bool TILE = false>
__device__ __forceinline__ int e_sweep(const StepParams& p, const float4* C4, const float* Cs,
                                       const float2* CD, int q, int base, int stride, int it,
                                       int lim = 0) {
  q -= base;
  lim -= base;   // TILE: positions from lim on belong to another block
  {
    const Box& B = p.boxE[0];
    const int end = B.start + B.count;
    if (q < end && (!TILE || q < lim)) {
      BoxWalk w(q - B.start, stride, B);
      for (; q < end && (!TILE || q < lim); q += stride, w.advance(B))
        e_site<PK, NP, IDP, true, TR>(p, C4, Cs, CD, B.i0 + w.a, B.j0 + w.b, w.k(B), it);
    }
  }
#pragma unroll 1
  for (int b = 1; b < kBoxes; ++b) {
    if (TILE && q >= lim) break;
    const Box& B = p.boxE[b];
    const int end = B.start + B.count;
    if (q >= end) continue;
    BoxWalk w(q - B.start, stride, B);
    for (; q < end && (!TILE || q < lim); q += stride, w.advance(B))
      e_site<PK, NP, IDP, false, TR>(p, C4, Cs, CD, B.i0 + w.a, B.j0 + w.b, w.k(B), it);
  }
  return q + base;
}

// Shared-memory layout of the E tables: float4 rows, srce column (padded to 16 bytes), then the
// dispersive coefficients (complex [nmat][3P], or with the real pole state float4 [nmat][P]).
__device__ __forceinline__ void e_tables(const StepParams& p, float4* smem, float4*& s4,
                                         float*& ss, float2*& sd) {
  s4 = smem;
  ss = reinterpret_cast<float*>(s4 + (p.smem ? p.nmat : 0));
  sd = reinterpret_cast<float2*>(ss + (p.smem ? ((p.nmat + 3) & ~3) : 0));   // 16-byte aligned
}

// TR: the dispersive state is stored as fp32 real parts ([3][P][ncomp] floats), possible when
// every pole's eqt has imaginary part +0 and zt imaginary part +-0 (Debye poles): the update
// then keeps every imaginary part at exactly +0 (it starts at +0, and each product and sum
// forming it is a signed zero that adds to +0), and the real parts are computed from the same
// operands as with the complex state, so the results are the same bit for bit.
template <int PK, int NP, int IDP, bool TR>
__global__ void __launch_bounds__(kThreads, NP >= 3 ? 3 : 4)
e_half_step(const __grid_constant__ StepParams p) {
  extern __shared__ float4 smem_e[];
  float4* s4;
  float* ss;
  float2* sd;
  e_tables(p, smem_e, s4, ss, sd);
  if (p.smem) {
    stage_tables(p, true, s4, ss, NP > 0 ? sd : nullptr);
    __syncthreads();
  }
  const float4* C4 = p.smem ? s4 : p.cE4;
  const float* Cs = p.smem ? ss : p.cEs;
  const float2* CD = (p.smem && NP > 0) ? sd : p.cD;
  int it = 0;
  if (p.nsrcE) it = *p.d_it;
  e_sweep<PK, NP, IDP, TR>(p, C4, Cs, CD, blockIdx.x * blockDim.x + threadIdx.x, 0,
                           gridDim.x * blockDim.x, it);
}

template <int PK, int NP, int IDP, bool TR>
__global__ void __launch_bounds__(kThreads, NP >= 3 ? 3 : 4)
e_half_step_batch(const __grid_constant__ BatchParams bp) {
  __shared__ StepParams p;
  extern __shared__ float4 smem_eb[];
  const int total = __ldg(bp.rangeE + bp.n);
  int m = 0, mend = -1;   // as h_half_step_batch
  int mbeg = 0, it = 0;
  const float4* C4 = nullptr;
  const float* Cs = nullptr;
  const float2* CD = nullptr;
#pragma unroll 1
  for (int t0 = blockIdx.x * kBatchTile; t0 < total; t0 += gridDim.x * kBatchTile) {
    if (t0 >= mend) {
      while (__ldg(bp.rangeE + m + 1) <= t0) ++m;
      mbeg = __ldg(bp.rangeE + m);
      mend = __ldg(bp.rangeE + m + 1);
      __syncthreads();
      load_params(p, bp.models + m);
      __syncthreads();
      float4* s4;
      float* ss;
      float2* sd;
      e_tables(p, smem_eb, s4, ss, sd);
      if (p.smem) stage_tables(p, true, s4, ss, NP > 0 ? sd : nullptr);
      __syncthreads();
      C4 = p.smem ? s4 : p.cE4;
      Cs = p.smem ? ss : p.cEs;
      CD = (p.smem && NP > 0) ? sd : p.cD;
      it = p.nsrcE ? *p.d_it : 0;
    }
    e_sweep<PK, NP, IDP, TR, true>(p, C4, Cs, CD, t0 + threadIdx.x, mbeg, blockDim.x, it,
                                   t0 + kBatchTile);
  }
}

#ifndef GBF_KERNELS_ONLY
// ---------------------------------------------------------------------------------------
// End of an iteration: electric sources on nodes outside the E kernel's domain, then the
// receiver samples that the next iteration starts from (fields_outputs.py:40-67, grid.py:
// 413-461), then the iteration counter advances.
// A transmission line attached to one E edge (sources.py:286-451). The connected line has
// antpos + 1 cells; its updates are the reference's numpy expressions, which evaluate in float64
// (the step ratios are float64 scalars) and round to float32 on assignment.
constexpr int kTLCells = 16;
struct TLine {
  int comp, i, j, k, first, last, nl, srcpos, antpos;
  float d;            // cell size along the edge (fp32)
  double s_iv;        // (1/R) c dt / dl
  double s_vi;        // R c dt / dl
  double r;           // c dt / dl
  double h;           // absorbing end: (c dt - dl) / (c dt + dl)
  float v[kTLCells];  // line voltage
  float c[kTLCells];  // line current
  float abcv0, abcv1;
  float eset;         // -V(antpos)/d for this iteration's E half-step
  const float* whole; // waveform at whole and half steps [iterations]
  const float* half;
};

struct RxParams {
  const float* Eold[3];  // E the step read (the other buffer after a fused step; else E itself)
  const int* coords;   // [nrx][3]
  float* out;          // [9][iterations][nrx]
  int nrx;
  int iterations;
  float dx, dy, dz;
  int nsrcOut;
  const Src* srcOut;
  const TLine* tls;    // [ntl]
  int ntl;
  float* tl_out;       // [ntl][2][iterations]: Vtotal, Itotal
};

__device__ __forceinline__ void end_of_step_body(const StepParams& p, const RxParams& r, int* d_it) {
  const int it = *d_it;
  if (threadIdx.x == 0) {
    // E outside the half-step's range changes only here: after a fused step, which wrote its
    // E into the other buffer, each source node first takes its value from the buffer the step
    // read, active or not, so that both buffers keep it
    for (int s = 0; s < r.nsrcOut; ++s) {
      const Src& q = r.srcOut[s];
      if (q.comp < 3 && r.Eold[q.comp] != p.E[q.comp]) {
        const long long idx = (long long)q.i * p.sx + (long long)q.j * p.sy + q.k;
        p.E[q.comp][idx] = r.Eold[q.comp][idx];
      }
    }
    for (int s = 0; s < r.nsrcOut; ++s) {
      const Src& q = r.srcOut[s];
      if (it < q.first || it > q.last) continue;
      const long long idx = (long long)q.i * p.sx + (long long)q.j * p.sy + q.k;
      float* E = p.E[q.comp];
      if (q.kind == 4) {
        E[idx] = *q.w;
        continue;
      }
      // the edge's material: from the packed E word, or the ID array when IDs are not packed
      const uint32_t m = p.PE ? (p.PE[idx] >> (kPackBits * q.comp)) & kPackMask : p.ID[q.comp][idx];
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
    for (int n = threadIdx.x; n < r.ntl; n += blockDim.x) {
      const TLine& t = r.tls[n];
      r.tl_out[(size_t)(2 * n) * r.iterations + sample] = t.v[t.antpos];
      r.tl_out[(size_t)(2 * n + 1) * r.iterations + sample] = t.c[t.antpos];
    }
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

// The current around an E edge (grid.py:413-461): Ix, Iy or Iz at node (x, y, z), fp32.
__device__ __forceinline__ float edge_current(const StepParams& p, int comp, int x, int y, int z,
                                              float dx, float dy, float dz) {
  const long long idx = (long long)x * p.sx + (long long)y * p.sy + z;
  const float* Hx = p.H[0];
  const float* Hy = p.H[1];
  const float* Hz = p.H[2];
  if (comp == 0)
    return (y == 0 || z == 0) ? 0.f :
        __fadd_rn(__fmul_rn(dy, __fsub_rn(Hy[idx - 1], Hy[idx])),
                  __fmul_rn(dz, __fsub_rn(Hz[idx], Hz[idx - p.sy])));
  if (comp == 1)
    return (x == 0 || z == 0) ? 0.f :
        __fadd_rn(__fmul_rn(dx, __fsub_rn(Hx[idx], Hx[idx - 1])),
                  __fmul_rn(dz, __fsub_rn(Hz[idx - p.sx], Hz[idx])));
  return (x == 0 || y == 0) ? 0.f :
      __fadd_rn(__fmul_rn(dx, __fsub_rn(Hx[idx - p.sy], Hx[idx])),
                __fmul_rn(dy, __fsub_rn(Hy[idx], Hy[idx - p.sx])));
}

// Transmission lines between the H and E half-steps (one thread per line): the magnetic part
// (update_current, then the line current at the antenna cell from the grid's H; sources.py:
// 426-451) and the voltage update of the electric part (update_voltage with its absorbing end;
// :396-424), whose -V/d the E half-step writes into the edge.
__global__ void tl_step(const __grid_constant__ StepParams p, TLine* tls, int ntl, float dx,
                        float dy, float dz) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= ntl) return;
  const int it = *p.d_it;
  TLine& t = tls[n];
  if (it < t.first || it > t.last) return;
  const int nl = t.nl;
  // current[0:nl-1] -= s_iv * (v[1:nl] - v[0:nl-1]); current[srcpos-1] += s_iv * half[it]
  for (int m = 0; m < nl - 1; ++m)
    t.c[m] = __double2float_rn(__dsub_rn((double)t.c[m], __dmul_rn(t.s_iv, (double)__fsub_rn(t.v[m + 1], t.v[m]))));
  t.c[t.srcpos - 1] = __double2float_rn(__dadd_rn((double)t.c[t.srcpos - 1], __dmul_rn(t.s_iv, (double)t.half[it])));
  t.c[t.antpos] = edge_current(p, t.comp, t.i, t.j, t.k, dx, dy, dz);
  // voltage[1:nl] -= s_vi * (c[1:nl] - c[0:nl-1]); voltage[srcpos] += r * whole[it]
  for (int m = nl - 1; m >= 1; --m)
    t.v[m] = __double2float_rn(__dsub_rn((double)t.v[m], __dmul_rn(t.s_vi, (double)__fsub_rn(t.c[m], t.c[m - 1]))));
  t.v[t.srcpos] = __double2float_rn(__dadd_rn((double)t.v[t.srcpos], __dmul_rn(t.r, (double)t.whole[it])));
  // absorbing end: v[0] = h (v[1] - abcv0) + abcv1
  t.v[0] = __double2float_rn(__dadd_rn(__dmul_rn(t.h, (double)__fsub_rn(t.v[1], t.abcv0)), (double)t.abcv1));
  t.abcv0 = t.v[0];
  t.abcv1 = t.v[1];
  t.eset = __fdiv_rn(-t.v[t.antpos], t.d);
}

__global__ void end_of_step(const __grid_constant__ StepParams p, const __grid_constant__ RxParams r, int* d_it) {
  end_of_step_body(p, r, d_it);
}

// The end of an iteration for every model of a batch: one block per model.
__global__ void end_of_step_batch(const StepParams* models, const RxParams* rxs) {
  __shared__ StepParams p;
  __shared__ RxParams r;
  load_params(p, models + blockIdx.x);
  if (threadIdx.x == 0) r = rxs[blockIdx.x];
  __syncthreads();
  end_of_step_body(p, r, const_cast<int*>(p.d_it));
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

#endif  // GBF_KERNELS_ONLY
}  // namespace gbf
