// geom.cu — model geometry built in device memory (part of libgbfdtd.so, see include/gbfdtd.h).
//
// The solid, rigid and per-edge material-ID arrays of a gprMax grid (gprMax/grid.py:157-169)
// live on the device while the geometry commands run, and the E/H component build with
// dielectric smoothing (gprMax/yee_cell_build_ext.pyx:110-257) completes the ID array there.
// The host resolves the averaged materials (their names and numbers are part of the model)
// from the list of neighbour combinations that the device compacts in the reference's loop
// order, and the solver takes the finished ID array without a round trip through the host.
//
// Device layout (C order, k fastest):
//   solid  uint32 [nx][ny][nz]            material number of each cell
//   rigid  uint32 [nx][ny][nz]            bits 0-11 rigidE[0..11], bits 12-17 rigidH[0..5]
//                                         (gprMax/yee_cell_setget_rigid_ext.pyx:24-157)
//   ID     uint32 [6][nx+1][ny+1][nz+1]   Ex Ey Ez Hx Hy Hz
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbfdtd.h"

namespace {

constexpr int kThreads = 256;
constexpr int kIters = 8;                        // edges per block pass = kIters * kThreads
constexpr long long kChunk = (long long)kIters * kThreads;
constexpr uint32_t kAllRigid = 0x3FFFFu;         // 12 E bits and 6 H bits

struct Dims {
  int nx, ny, nz;
  long long ncell, nnode;
};

__device__ __forceinline__ long long cell_at(const Dims& d, int i, int j, int k) {
  return ((long long)i * d.ny + j) * d.nz + k;
}
__device__ __forceinline__ long long node_at(const Dims& d, int i, int j, int k) {
  return ((long long)i * (d.ny + 1) + j) * (d.nz + 1) + k;
}

// ---- primitives ---------------------------------------------------------------------------

// build_voxel (geometry_primitives_ext.pyx:314-377) for every selected cell of a box: one
// material, so cells sharing an edge write the same value and their order does not matter.
__global__ void cells_kernel(Dims d, int xs, int ys, int zs, int sx, int sy, int sz,
                             const uint8_t* mask, uint32_t numID, uint32_t vx, uint32_t vy,
                             uint32_t vz, int averaging, int edges, uint32_t* solid,
                             uint32_t* rigid, uint32_t* ID) {
  const long long n = (long long)sx * sy * sz;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    if (mask && !mask[q]) continue;
    const int k = zs + (int)(q % sz);
    const long long t = q / sz;
    const int j = ys + (int)(t % sy);
    const int i = xs + (int)(t / sy);
    const long long c = cell_at(d, i, j, k);
    solid[c] = numID;
    rigid[c] = averaging ? 0u : kAllRigid;
    if (averaging || !edges) continue;
    uint32_t* X = ID;
    uint32_t* Y = ID + d.nnode;
    uint32_t* Z = ID + 2 * d.nnode;
    X[node_at(d, i, j, k)] = vx;
    X[node_at(d, i, j + 1, k + 1)] = vx;
    X[node_at(d, i, j + 1, k)] = vx;
    X[node_at(d, i, j, k + 1)] = vx;
    Y[node_at(d, i, j, k)] = vy;
    Y[node_at(d, i + 1, j, k + 1)] = vy;
    Y[node_at(d, i + 1, j, k)] = vy;
    Y[node_at(d, i, j, k + 1)] = vy;
    Z[node_at(d, i, j, k)] = vz;
    Z[node_at(d, i + 1, j + 1, k)] = vz;
    Z[node_at(d, i + 1, j, k)] = vz;
    Z[node_at(d, i, j + 1, k)] = vz;
    uint32_t* HX = ID + 3 * d.nnode;
    uint32_t* HY = ID + 4 * d.nnode;
    uint32_t* HZ = ID + 5 * d.nnode;
    HX[node_at(d, i, j, k)] = vx;
    HX[node_at(d, i, j + 1, k + 1)] = vx;
    HX[node_at(d, i, j + 1, k)] = vx;
    HX[node_at(d, i, j, k + 1)] = vx;
    HY[node_at(d, i, j, k)] = vy;
    HY[node_at(d, i + 1, j, k + 1)] = vy;
    HY[node_at(d, i + 1, j, k)] = vy;
    HY[node_at(d, i, j, k + 1)] = vy;
    HZ[node_at(d, i, j, k)] = vz;
    HZ[node_at(d, i + 1, j + 1, k)] = vz;
    HZ[node_at(d, i + 1, j, k)] = vz;
    HZ[node_at(d, i, j + 1, k)] = vz;
  }
}

// build_box's ID ranges (geometry_primitives_ext.pyx:660-690): per component a node range that
// differs from the union of the cells' build_voxel edges (the H components in particular).
__global__ void box_ids_kernel(Dims d, int xs, int ys, int zs, int sx, int sy, int sz,
                               uint32_t vx, uint32_t vy, uint32_t vz, uint32_t* ID) {
  const int ex = sx + 1, ey = sy + 1, ez = sz + 1;
  const long long n = (long long)ex * ey * ez;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const int c = (int)(q % ez);
    const long long t = q / ez;
    const int b = (int)(t % ey);
    const int a = (int)(t / ey);
    const bool ia = a < sx, jb = b < sy, kc = c < sz;   // inside the half-open cell range
    const long long node = node_at(d, xs + a, ys + b, zs + c);
    if (ia) ID[node] = vx;                                  // Ex: i < xf, j <= yf, k <= zf
    if (jb) ID[d.nnode + node] = vy;                        // Ey
    if (kc) ID[2 * d.nnode + node] = vz;                    // Ez
    if (jb && kc) ID[3 * d.nnode + node] = vx;              // Hx: i <= xf, j < yf, k < zf
    if (ia && kc) ID[4 * d.nnode + node] = vy;              // Hy
    if (ia && jb) ID[5 * d.nnode + node] = vz;              // Hz
  }
}

// build_voxels_from_array (geometry_primitives_ext.pyx:934-980), cell part: solid and rigid of
// every cell whose value is not negative.
__global__ void voxel_cells_kernel(Dims d, int xs, int ys, int zs, int sx, int sy, int sz,
                                   const int16_t* data, int numexist, int averaging,
                                   uint32_t* solid, uint32_t* rigid) {
  const long long n = (long long)sx * sy * sz;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const int v = data[q];
    if (v < 0) continue;
    const int k = zs + (int)(q % sz);
    const long long t = q / sz;
    const int j = ys + (int)(t % sy);
    const int i = xs + (int)(t / sy);
    const long long c = cell_at(d, i, j, k);
    solid[c] = (uint32_t)(numexist + v);
    rigid[c] = averaging ? 0u : kAllRigid;
  }
}

// Edge part: the cells of a voxel block write shared edges in the reference's (i, j, k) loop
// order, so an edge keeps the value of the last built cell among those touching it. Each node
// of the block's node range looks at its candidate cells latest first.
__device__ __forceinline__ int voxel_value(int xs, int ys, int zs, int sx, int sy, int sz,
                                           const int16_t* data, int i, int j, int k) {
  const int a = i - xs, b = j - ys, c = k - zs;
  if (a < 0 || b < 0 || c < 0 || a >= sx || b >= sy || c >= sz) return -1;
  return data[((long long)a * sy + b) * sz + c];
}

__global__ void voxel_edges_kernel(Dims d, int xs, int ys, int zs, int sx, int sy, int sz,
                                   const int16_t* data, int numexist, uint32_t* ID) {
  // candidate cells (node minus offset), latest in loop order first, per component
  const int off[3][4][3] = {{{0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1}},
                            {{0, 0, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 1}},
                            {{0, 0, 0}, {0, 1, 0}, {1, 0, 0}, {1, 1, 0}}};
  const int ex = sx + 1, ey = sy + 1, ez = sz + 1;
  const long long n = (long long)ex * ey * ez;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const int k = zs + (int)(q % ez);
    const long long t = q / ez;
    const int j = ys + (int)(t % ey);
    const int i = xs + (int)(t / ey);
    if (i > d.nx || j > d.ny || k > d.nz) continue;
    const long long node = node_at(d, i, j, k);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        const int v = voxel_value(xs, ys, zs, sx, sy, sz, data, i - off[comp][o][0],
                                  j - off[comp][o][1], k - off[comp][o][2]);
        if (v >= 0) {
          ID[comp * d.nnode + node] = (uint32_t)(numexist + v);
          ID[(comp + 3) * d.nnode + node] = (uint32_t)(numexist + v);
          break;
        }
      }
    }
  }
}

// Rigid single edges with their material (set_rigid_Ex/Ey/Ez, yee_cell_setget_rigid_ext.pyx
// :72-97, and the ID write of #edge / #plate). recs: n x 5 (component 0..2, i, j, k, value).
__global__ void edges_kernel(Dims d, int n, const int32_t* recs, uint32_t* rigid, uint32_t* ID) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int32_t* r = recs + 5 * (long long)q;
    const int comp = r[0], i = r[1], j = r[2], k = r[3];
    const uint32_t v = (uint32_t)r[4];
    if (comp == 0) {
      atomicOr(&rigid[cell_at(d, i, j, k)], 1u << 0);
      if (j != 0) atomicOr(&rigid[cell_at(d, i, j - 1, k)], 1u << 1);
      if (k != 0) atomicOr(&rigid[cell_at(d, i, j, k - 1)], 1u << 3);
      if (j != 0 && k != 0) atomicOr(&rigid[cell_at(d, i, j - 1, k - 1)], 1u << 2);
    } else if (comp == 1) {
      atomicOr(&rigid[cell_at(d, i, j, k)], 1u << 4);
      if (i != 0) atomicOr(&rigid[cell_at(d, i - 1, j, k)], 1u << 7);
      if (k != 0) atomicOr(&rigid[cell_at(d, i, j, k - 1)], 1u << 5);
      if (i != 0 && k != 0) atomicOr(&rigid[cell_at(d, i - 1, j, k - 1)], 1u << 6);
    } else {
      atomicOr(&rigid[cell_at(d, i, j, k)], 1u << 8);
      if (i != 0) atomicOr(&rigid[cell_at(d, i - 1, j, k)], 1u << 9);
      if (j != 0) atomicOr(&rigid[cell_at(d, i, j - 1, k)], 1u << 11);
      if (i != 0 && j != 0) atomicOr(&rigid[cell_at(d, i - 1, j - 1, k)], 1u << 10);
    }
    ID[comp * d.nnode + node_at(d, i, j, k)] = v;
  }
}

__global__ void fill_kernel(Dims d, uint32_t* arr, int ry, int rz, int xs, int ys, int zs,
                            int sx, int sy, int sz, uint32_t value) {
  const long long n = (long long)sx * sy * sz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int k = zs + (int)(q % sz);
    const long long t = q / sz;
    const int j = ys + (int)(t % sy);
    const int i = xs + (int)(t / sy);
    arr[((long long)i * ry + j) * rz + k] = value;
  }
}

__global__ void gather_kernel(const uint32_t* arr, int ry, int rz, int xs, int ys, int zs, int sx,
                              int sy, int sz, uint32_t* out) {
  const long long n = (long long)sx * sy * sz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int k = zs + (int)(q % sz);
    const long long t = q / sz;
    const int j = ys + (int)(t % sy);
    const int i = xs + (int)(t / sy);
    out[q] = arr[((long long)i * ry + j) * rz + k];
  }
}

// ---- E/H component build (yee_cell_build_ext.pyx:110-257) ----------------------------------

// One component's build: its node range, its neighbour cells (node minus offset, in the order
// their materials enter an averaged material's name) and the rigid bits that exclude an edge.
struct Comp {
  int comp;
  int i0, j0, k0, ri, rj, rk;
  int nnb;
  int nb[4][3];
  int rbit[4];
  int rof[4][3];
};

// 0: rigid (left as written by the primitives), 1: one material (*value), 2: averaged (*key)
__device__ __forceinline__ int classify(const Dims& d, const Comp& c, const uint32_t* solid,
                                        const uint32_t* rigid, long long r, long long* node,
                                        uint32_t* value, unsigned long long* key) {
  const int k = c.k0 + (int)(r % c.rk);
  const long long t = r / c.rk;
  const int j = c.j0 + (int)(t % c.rj);
  const int i = c.i0 + (int)(t / c.rj);
  *node = node_at(d, i, j, k);
  uint32_t rig = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < c.nnb) rig |= rigid[cell_at(d, i - c.rof[q][0], j - c.rof[q][1], k - c.rof[q][2])] & (1u << c.rbit[q]);
  if (rig) return 0;
  uint32_t s[4] = {0, 0, 0, 0};
  bool same = true;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < c.nnb) {
      s[q] = solid[cell_at(d, i - c.nb[q][0], j - c.nb[q][1], k - c.nb[q][2])];
      same = same && s[q] == s[0];
    }
  if (same) {
    *value = s[0];
    return 1;
  }
  if (c.nnb == 4)
    *key = ((unsigned long long)s[0] << 48) | ((unsigned long long)s[1] << 32) |
           ((unsigned long long)s[2] << 16) | (unsigned long long)s[3];
  else
    *key = ((unsigned long long)s[0] << 16) | (unsigned long long)s[1];
  return 2;
}

// Pass 1: write the one-material edges and count the averaged ones of each chunk.
__global__ void comp_count_kernel(Dims d, Comp c, const uint32_t* solid, const uint32_t* rigid,
                                  uint32_t* ID, unsigned int* counts) {
  __shared__ unsigned int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const long long R = (long long)c.ri * c.rj * c.rk;
  const long long base = blockIdx.x * kChunk;
  unsigned int mine = 0;
  for (int it = 0; it < kIters; ++it) {
    const long long r = base + (long long)it * kThreads + threadIdx.x;
    if (r >= R) break;
    long long node;
    uint32_t v;
    unsigned long long key;
    const int kind = classify(d, c, solid, rigid, r, &node, &v, &key);
    if (kind == 1) ID[c.comp * d.nnode + node] = v;
    mine += kind == 2;
  }
  if (mine) atomicAdd(&total, mine);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// Exclusive prefix sum of the chunk counts (one block), total in out[n].
__global__ void scan_kernel(const unsigned int* counts, long long n, unsigned long long* out) {
  __shared__ unsigned long long part[1024];
  const long long per = (n + blockDim.x - 1) / blockDim.x;
  const long long lo = threadIdx.x * per;
  const long long hi = lo + per < n ? lo + per : n;
  unsigned long long s = 0;
  for (long long q = lo; q < hi; ++q) s += counts[q];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (int q = 0; q < (int)blockDim.x; ++q) {
      const unsigned long long v = part[q];
      part[q] = run;
      run += v;
    }
    out[n] = run;
  }
  __syncthreads();
  unsigned long long run = part[threadIdx.x];
  for (long long q = lo; q < hi; ++q) {
    out[q] = run;
    run += counts[q];
  }
}

// Pass 2: write each averaged edge's key and position at its rank in loop order.
__global__ void comp_scatter_kernel(Dims d, Comp c, const uint32_t* solid, const uint32_t* rigid,
                                    const unsigned long long* offsets, unsigned long long base_out,
                                    unsigned long long* keys, unsigned long long* pos) {
  __shared__ unsigned int warp_tot[kThreads / 32];
  const long long R = (long long)c.ri * c.rj * c.rk;
  const long long base = blockIdx.x * kChunk;
  unsigned long long out = base_out + offsets[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int it = 0; it < kIters; ++it) {
    const long long r = base + (long long)it * kThreads + threadIdx.x;
    long long node = 0;
    uint32_t v;
    unsigned long long key = 0;
    const int kind = r < R ? classify(d, c, solid, rigid, r, &node, &v, &key) : 0;
    const unsigned int ballot = __ballot_sync(0xffffffffu, kind == 2);
    if (lane == 0) warp_tot[warp] = __popc(ballot);
    __syncthreads();
    unsigned int before = 0, all = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      before += w < warp ? warp_tot[w] : 0;
      all += warp_tot[w];
    }
    if (kind == 2) {
      const unsigned long long at = out + before + __popc(ballot & ((1u << lane) - 1u));
      keys[at] = key;
      pos[at] = (unsigned long long)c.comp * d.nnode + node;
    }
    out += all;
    __syncthreads();
  }
}

// Averaged edges take the number the host resolved for their key (table sorted by key).
__global__ void resolve_kernel(long long n, const unsigned long long* keys,
                               const unsigned long long* pos, long long m,
                               const unsigned long long* table, const uint32_t* numbers,
                               uint32_t* ID, int* missing) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const unsigned long long key = keys[q];
    long long lo = 0, hi = m;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (table[mid] < key) lo = mid + 1;
      else hi = mid;
    }
    if (lo < m && table[lo] == key) ID[pos[q]] = numbers[lo];
    else atomicExch(missing, 1);
  }
}

__global__ void max_kernel(const uint32_t* a, long long n, unsigned int* mx) {
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

__global__ void init_kernel(uint32_t* solid, uint32_t* rigid, long long ncell, uint32_t* ID,
                            long long nid) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ncell; q += stride) {
    solid[q] = 1u;
    rigid[q] = 0u;
  }
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nid; q += stride)
    ID[q] = 1u;
}

}  // namespace

struct gbf_geom {
  Dims d{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  uint32_t* solid = nullptr;
  uint32_t* rigid = nullptr;
  uint32_t* ID = nullptr;
  int grid = 0;                            // blocks of the grid-stride kernels
  // the averaged edges of the last gbf_geom_components call
  unsigned long long* keys = nullptr;
  unsigned long long* pos = nullptr;
  long long navg = 0;
  int avg_electric = -1;
};

namespace gbf {
// Device ID array and grid size of a geometry, for gbf_upload_materials_geom.
const uint32_t* geom_ids(const gbf_geom* g, int dims[3], int* device, cudaStream_t* stream) {
  dims[0] = g->d.nx;
  dims[1] = g->d.ny;
  dims[2] = g->d.nz;
  *device = g->device;
  *stream = g->stream;
  return g->ID;
}
}  // namespace gbf

static std::string g_geom_err;

static int gfail(gbf_geom* g, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  (g ? g->err : g_geom_err) = buf;
  return code;
}

#define GK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return gfail(g, e_ == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA, "%s: %s",   \
                   #call, cudaGetErrorString(e_));                                          \
  } while (0)

static int blocks_for(const gbf_geom* g, long long n) {
  const long long b = (n + kThreads - 1) / kThreads;
  return (int)(b < g->grid ? (b > 0 ? b : 1) : g->grid);
}

// box = xs, ys, zs, sx, sy, sz (cells); must lie in the grid
static bool box_ok(const gbf_geom* g, const int32_t* b) {
  return b && b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && b[3] > 0 && b[4] > 0 && b[5] > 0 &&
         b[0] + b[3] <= g->d.nx && b[1] + b[4] <= g->d.ny && b[2] + b[5] <= g->d.nz;
}

static void free_avg(gbf_geom* g) {
  if (g->keys) cudaFree(g->keys);
  if (g->pos) cudaFree(g->pos);
  g->keys = nullptr;
  g->pos = nullptr;
  g->navg = 0;
  g->avg_electric = -1;
}

extern "C" {

int gbf_geom_create(int32_t nx, int32_t ny, int32_t nz, gbf_geom** out) {
  if (!out) return GBF_EINVAL;
  *out = nullptr;
  gbf_geom* g = nullptr;
  if (nx < 1 || ny < 1 || nz < 1) return gfail(g, GBF_EINVAL, "gbf_geom_create: bad grid %d x %d x %d", nx, ny, nz);
  g = new gbf_geom();
  g->d.nx = nx;
  g->d.ny = ny;
  g->d.nz = nz;
  g->d.ncell = (long long)nx * ny * nz;
  g->d.nnode = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  int rc = GBF_OK;
  auto A = [&](uint32_t** p, long long n) {
    if (rc != GBF_OK) return;
    cudaError_t e = cudaMalloc((void**)p, sizeof(uint32_t) * (size_t)n);
    if (e != cudaSuccess)
      rc = gfail(g, e == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA,
                 "gbf_geom_create: allocation of %lld bytes failed: %s", 4 * n, cudaGetErrorString(e));
  };
  cudaError_t e = cudaGetDevice(&g->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) rc = gfail(g, GBF_ECUDA, "gbf_geom_create: %s", cudaGetErrorString(e));
  A(&g->solid, g->d.ncell);
  A(&g->rigid, g->d.ncell);
  A(&g->ID, 6 * g->d.nnode);
  if (rc == GBF_OK) {
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device);
    g->grid = sms * 8;
    init_kernel<<<g->grid, kThreads, 0, g->stream>>>(g->solid, g->rigid, g->d.ncell, g->ID, 6 * g->d.nnode);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) rc = gfail(g, GBF_ECUDA, "gbf_geom_create: %s", cudaGetErrorString(e));
  }
  if (rc != GBF_OK) {
    g_geom_err = g->err;
    gbf_geom_destroy(g);
    return rc;
  }
  *out = g;
  return GBF_OK;
}

void gbf_geom_destroy(gbf_geom* g) {
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  free_avg(g);
  if (g->solid) cudaFree(g->solid);
  if (g->rigid) cudaFree(g->rigid);
  if (g->ID) cudaFree(g->ID);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

int gbf_geom_last_error(gbf_geom* g, char* buf, size_t n) {
  if (!buf || n == 0) return GBF_EINVAL;
  snprintf(buf, n, "%s", g ? g->err.c_str() : g_geom_err.c_str());
  return GBF_OK;
}

int gbf_geom_cells(gbf_geom* g, const int32_t box[6], const uint8_t* mask, const uint32_t num[4],
                   int32_t averaging) {
  if (!g || !num) return GBF_EINVAL;
  if (!box_ok(g, box)) return gfail(g, GBF_EINVAL, "gbf_geom_cells: box outside the grid");
  const long long n = (long long)box[3] * box[4] * box[5];
  uint8_t* dmask = nullptr;
  if (mask) {
    GK(cudaMallocAsync((void**)&dmask, (size_t)n, g->stream));
    GK(cudaMemcpyAsync(dmask, mask, (size_t)n, cudaMemcpyHostToDevice, g->stream));
  }
  cells_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(
      g->d, box[0], box[1], box[2], box[3], box[4], box[5], dmask, num[0], num[1], num[2], num[3],
      averaging ? 1 : 0, 1, g->solid, g->rigid, g->ID);
  GK(cudaGetLastError());
  if (dmask) GK(cudaFreeAsync(dmask, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_box(gbf_geom* g, const int32_t box[6], const uint32_t num[4], int32_t averaging) {
  if (!g || !num) return GBF_EINVAL;
  if (!box_ok(g, box)) return gfail(g, GBF_EINVAL, "gbf_geom_box: box outside the grid");
  const long long n = (long long)box[3] * box[4] * box[5];
  cells_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(
      g->d, box[0], box[1], box[2], box[3], box[4], box[5], nullptr, num[0], num[1], num[2],
      num[3], averaging ? 1 : 0, 0, g->solid, g->rigid, g->ID);
  GK(cudaGetLastError());
  if (!averaging) {
    const long long ne = (long long)(box[3] + 1) * (box[4] + 1) * (box[5] + 1);
    box_ids_kernel<<<blocks_for(g, ne), kThreads, 0, g->stream>>>(
        g->d, box[0], box[1], box[2], box[3], box[4], box[5], num[1], num[2], num[3], g->ID);
    GK(cudaGetLastError());
  }
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_voxels(gbf_geom* g, const int32_t box[6], const int16_t* data, int32_t numexist,
                    int32_t averaging) {
  if (!g || !data) return GBF_EINVAL;
  if (!box_ok(g, box)) return gfail(g, GBF_EINVAL, "gbf_geom_voxels: block outside the grid");
  const long long n = (long long)box[3] * box[4] * box[5];
  int16_t* dd = nullptr;
  GK(cudaMallocAsync((void**)&dd, sizeof(int16_t) * (size_t)n, g->stream));
  GK(cudaMemcpyAsync(dd, data, sizeof(int16_t) * (size_t)n, cudaMemcpyHostToDevice, g->stream));
  voxel_cells_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(
      g->d, box[0], box[1], box[2], box[3], box[4], box[5], dd, numexist, averaging ? 1 : 0,
      g->solid, g->rigid);
  GK(cudaGetLastError());
  if (!averaging) {
    const long long ne = (long long)(box[3] + 1) * (box[4] + 1) * (box[5] + 1);
    voxel_edges_kernel<<<blocks_for(g, ne), kThreads, 0, g->stream>>>(
        g->d, box[0], box[1], box[2], box[3], box[4], box[5], dd, numexist, g->ID);
    GK(cudaGetLastError());
  }
  GK(cudaFreeAsync(dd, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_edges(gbf_geom* g, int32_t n, const int32_t* recs) {
  if (!g || n < 0 || (n > 0 && !recs)) return GBF_EINVAL;
  for (int32_t q = 0; q < n; ++q) {
    const int32_t* r = recs + 5 * (size_t)q;
    if (r[0] < 0 || r[0] > 2 || r[1] < 0 || r[2] < 0 || r[3] < 0 || r[1] >= g->d.nx ||
        r[2] >= g->d.ny || r[3] >= g->d.nz || r[4] < 0)
      return gfail(g, GBF_EINVAL, "gbf_geom_edges: record %d (%d, %d, %d, %d) outside the grid", q,
                   r[0], r[1], r[2], r[3]);
  }
  if (n == 0) return GBF_OK;
  int32_t* dr = nullptr;
  GK(cudaMallocAsync((void**)&dr, sizeof(int32_t) * 5 * (size_t)n, g->stream));
  GK(cudaMemcpyAsync(dr, recs, sizeof(int32_t) * 5 * (size_t)n, cudaMemcpyHostToDevice, g->stream));
  edges_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(g->d, n, dr, g->rigid, g->ID);
  GK(cudaGetLastError());
  GK(cudaFreeAsync(dr, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_components(gbf_geom* g, int32_t electric, int64_t counts[3]) {
  if (!g || !counts) return GBF_EINVAL;
  free_avg(g);
  const Dims& d = g->d;
  Comp cs[3];
  for (int q = 0; q < 3; ++q) memset(&cs[q], 0, sizeof(Comp));
  if (electric) {
    // Ex: i [0,nx), j [1,ny), k [1,nz); cells (i,j,k) (i,j-1,k) (i,j-1,k-1) (i,j,k-1)
    cs[0] = Comp{0, 0, 1, 1, d.nx, d.ny - 1, d.nz - 1, 4,
                 {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}}, {0, 1, 3, 2},
                 {{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}}};
    // Ey: i [1,nx), j [0,ny), k [1,nz); cells (i,j,k) (i-1,j,k) (i-1,j,k-1) (i,j,k-1)
    cs[1] = Comp{1, 1, 0, 1, d.nx - 1, d.ny, d.nz - 1, 4,
                 {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}}, {4, 7, 5, 6},
                 {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}}};
    // Ez: i [1,nx), j [1,ny), k [0,nz); cells (i,j,k) (i-1,j,k) (i-1,j-1,k) (i,j-1,k)
    cs[2] = Comp{2, 1, 1, 0, d.nx - 1, d.ny - 1, d.nz, 4,
                 {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}}, {8, 9, 11, 10},
                 {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}}};
  } else {
    // Hx: i [1,nx), j [0,ny), k [0,nz); cells (i,j,k) (i-1,j,k)
    cs[0] = Comp{3, 1, 0, 0, d.nx - 1, d.ny, d.nz, 2, {{0, 0, 0}, {1, 0, 0}}, {12, 13},
                 {{0, 0, 0}, {1, 0, 0}}};
    // Hy: i [0,nx), j [1,ny), k [0,nz); cells (i,j,k) (i,j-1,k)
    cs[1] = Comp{4, 0, 1, 0, d.nx, d.ny - 1, d.nz, 2, {{0, 0, 0}, {0, 1, 0}}, {14, 15},
                 {{0, 0, 0}, {0, 1, 0}}};
    // Hz: i [0,nx), j [0,ny), k [1,nz); cells (i,j,k) (i,j,k-1)
    cs[2] = Comp{5, 0, 0, 1, d.nx, d.ny, d.nz - 1, 2, {{0, 0, 0}, {0, 0, 1}}, {16, 17},
                 {{0, 0, 0}, {0, 0, 1}}};
  }
  // averaged keys hold 16 bits per material number
  unsigned int* dmax = nullptr;
  GK(cudaMallocAsync((void**)&dmax, sizeof(unsigned int), g->stream));
  GK(cudaMemsetAsync(dmax, 0, sizeof(unsigned int), g->stream));
  max_kernel<<<blocks_for(g, d.ncell), kThreads, 0, g->stream>>>(g->solid, d.ncell, dmax);
  unsigned int smax = 0;
  GK(cudaMemcpyAsync(&smax, dmax, sizeof smax, cudaMemcpyDeviceToHost, g->stream));
  GK(cudaFreeAsync(dmax, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  if (smax > 0xFFFFu)
    return gfail(g, GBF_EINVAL, "gbf_geom_components: material number %u needs more than 16 bits", smax);

  unsigned int* cnt[3] = {nullptr, nullptr, nullptr};
  unsigned long long* off[3] = {nullptr, nullptr, nullptr};
  long long nb[3] = {0, 0, 0};
  unsigned long long tot[3] = {0, 0, 0};
  int rc = GBF_OK;
  for (int q = 0; q < 3 && rc == GBF_OK; ++q) {
    const long long R = (long long)cs[q].ri * cs[q].rj * cs[q].rk;
    if (cs[q].ri <= 0 || cs[q].rj <= 0 || cs[q].rk <= 0) continue;
    nb[q] = (R + kChunk - 1) / kChunk;
    cudaError_t e = cudaMallocAsync((void**)&cnt[q], sizeof(unsigned int) * nb[q], g->stream);
    if (e == cudaSuccess)
      e = cudaMallocAsync((void**)&off[q], sizeof(unsigned long long) * (nb[q] + 1), g->stream);
    if (e != cudaSuccess) {
      rc = gfail(g, GBF_ENOMEM, "gbf_geom_components: %s", cudaGetErrorString(e));
      break;
    }
    // nb[q] blocks of one chunk each (a grid of up to 2^31 - 1 blocks)
    comp_count_kernel<<<(unsigned)nb[q], kThreads, 0, g->stream>>>(d, cs[q], g->solid, g->rigid, g->ID, cnt[q]);
    scan_kernel<<<1, 1024, 0, g->stream>>>(cnt[q], nb[q], off[q]);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&tot[q], off[q] + nb[q], sizeof(unsigned long long), cudaMemcpyDeviceToHost, g->stream);
    if (e != cudaSuccess) rc = gfail(g, GBF_ECUDA, "gbf_geom_components: %s", cudaGetErrorString(e));
  }
  if (rc == GBF_OK) {
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) rc = gfail(g, GBF_ECUDA, "gbf_geom_components: %s", cudaGetErrorString(e));
  }
  const long long navg = (long long)(tot[0] + tot[1] + tot[2]);
  if (rc == GBF_OK && navg > 0) {
    cudaError_t e = cudaMalloc((void**)&g->keys, sizeof(unsigned long long) * navg);
    if (e == cudaSuccess) e = cudaMalloc((void**)&g->pos, sizeof(unsigned long long) * navg);
    if (e != cudaSuccess) {
      rc = gfail(g, GBF_ENOMEM, "gbf_geom_components: %lld averaged edges: %s", navg, cudaGetErrorString(e));
    } else {
      unsigned long long base = 0;
      for (int q = 0; q < 3; ++q) {
        if (nb[q] && tot[q])
          comp_scatter_kernel<<<(unsigned)nb[q], kThreads, 0, g->stream>>>(
              d, cs[q], g->solid, g->rigid, off[q], base, g->keys, g->pos);
        base += tot[q];
      }
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
      if (e != cudaSuccess) rc = gfail(g, GBF_ECUDA, "gbf_geom_components: %s", cudaGetErrorString(e));
    }
  }
  for (int q = 0; q < 3; ++q) {
    if (cnt[q]) cudaFreeAsync(cnt[q], g->stream);
    if (off[q]) cudaFreeAsync(off[q], g->stream);
  }
  cudaStreamSynchronize(g->stream);
  if (rc != GBF_OK) {
    free_avg(g);
    return rc;
  }
  g->navg = navg;
  g->avg_electric = electric ? 1 : 0;
  for (int q = 0; q < 3; ++q) counts[q] = (int64_t)tot[q];
  return GBF_OK;
}

int gbf_geom_averaged_keys(gbf_geom* g, uint64_t* keys) {
  if (!g || (!keys && g->navg)) return GBF_EINVAL;
  if (g->avg_electric < 0) return gfail(g, GBF_ESTATE, "gbf_geom_averaged_keys: run gbf_geom_components first");
  if (g->navg)
    GK(cudaMemcpy(keys, g->keys, sizeof(uint64_t) * (size_t)g->navg, cudaMemcpyDeviceToHost));
  return GBF_OK;
}

int gbf_geom_resolve(gbf_geom* g, int64_t m, const uint64_t* table, const uint32_t* numbers) {
  if (!g || m < 0 || (m > 0 && (!table || !numbers))) return GBF_EINVAL;
  if (g->avg_electric < 0) return gfail(g, GBF_ESTATE, "gbf_geom_resolve: run gbf_geom_components first");
  for (int64_t q = 1; q < m; ++q)
    if (!(table[q - 1] < table[q])) return gfail(g, GBF_EINVAL, "gbf_geom_resolve: table not strictly increasing at %lld", (long long)q);
  if (g->navg) {
    unsigned long long* dt = nullptr;
    uint32_t* dn = nullptr;
    int* miss = nullptr;
    GK(cudaMallocAsync((void**)&dt, sizeof(uint64_t) * (size_t)(m ? m : 1), g->stream));
    GK(cudaMallocAsync((void**)&dn, sizeof(uint32_t) * (size_t)(m ? m : 1), g->stream));
    GK(cudaMallocAsync((void**)&miss, sizeof(int), g->stream));
    if (m) {
      GK(cudaMemcpyAsync(dt, table, sizeof(uint64_t) * (size_t)m, cudaMemcpyHostToDevice, g->stream));
      GK(cudaMemcpyAsync(dn, numbers, sizeof(uint32_t) * (size_t)m, cudaMemcpyHostToDevice, g->stream));
    }
    GK(cudaMemsetAsync(miss, 0, sizeof(int), g->stream));
    resolve_kernel<<<blocks_for(g, g->navg), kThreads, 0, g->stream>>>(g->navg, g->keys, g->pos, m, dt, dn, g->ID, miss);
    GK(cudaGetLastError());
    int h_miss = 0;
    GK(cudaMemcpyAsync(&h_miss, miss, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    GK(cudaFreeAsync(dt, g->stream));
    GK(cudaFreeAsync(dn, g->stream));
    GK(cudaFreeAsync(miss, g->stream));
    GK(cudaStreamSynchronize(g->stream));
    if (h_miss) return gfail(g, GBF_EINVAL, "gbf_geom_resolve: an averaged edge's key is not in the table");
  }
  free_avg(g);
  return GBF_OK;
}

// array: 0 solid, 1 rigid, 2 + c: ID component c (0..5); box in that array's index space
static int array_of(gbf_geom* g, int32_t array, uint32_t** p, int* rx, int* ry, int* rz) {
  const Dims& d = g->d;
  if (array == 0 || array == 1) {
    *p = array == 0 ? g->solid : g->rigid;
    *rx = d.nx;
    *ry = d.ny;
    *rz = d.nz;
    return 1;
  }
  if (array >= 2 && array < 8) {
    *p = g->ID + (array - 2) * d.nnode;
    *rx = d.nx + 1;
    *ry = d.ny + 1;
    *rz = d.nz + 1;
    return 1;
  }
  return 0;
}

static bool sub_ok(const int32_t* b, int rx, int ry, int rz) {
  return b && b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && b[3] > 0 && b[4] > 0 && b[5] > 0 &&
         b[0] + b[3] <= rx && b[1] + b[4] <= ry && b[2] + b[5] <= rz;
}

int gbf_geom_fill(gbf_geom* g, int32_t array, const int32_t box[6], uint32_t value) {
  if (!g) return GBF_EINVAL;
  uint32_t* p;
  int rx, ry, rz;
  if (!array_of(g, array, &p, &rx, &ry, &rz)) return gfail(g, GBF_EINVAL, "gbf_geom_fill: bad array %d", array);
  if (!sub_ok(box, rx, ry, rz)) return gfail(g, GBF_EINVAL, "gbf_geom_fill: box outside the array");
  const long long n = (long long)box[3] * box[4] * box[5];
  fill_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(g->d, p, ry, rz, box[0], box[1], box[2],
                                                            box[3], box[4], box[5], value);
  GK(cudaGetLastError());
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_read(gbf_geom* g, int32_t array, const int32_t box[6], uint32_t* out) {
  if (!g || !out) return GBF_EINVAL;
  uint32_t* p;
  int rx, ry, rz;
  if (!array_of(g, array, &p, &rx, &ry, &rz)) return gfail(g, GBF_EINVAL, "gbf_geom_read: bad array %d", array);
  if (!sub_ok(box, rx, ry, rz)) return gfail(g, GBF_EINVAL, "gbf_geom_read: box outside the array");
  const long long n = (long long)box[3] * box[4] * box[5];
  uint32_t* tmp = nullptr;
  GK(cudaMallocAsync((void**)&tmp, sizeof(uint32_t) * (size_t)n, g->stream));
  gather_kernel<<<blocks_for(g, n), kThreads, 0, g->stream>>>(p, ry, rz, box[0], box[1], box[2],
                                                              box[3], box[4], box[5], tmp);
  GK(cudaGetLastError());
  GK(cudaMemcpyAsync(out, tmp, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost, g->stream));
  GK(cudaFreeAsync(tmp, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

int gbf_geom_max_id(gbf_geom* g, uint32_t* out) {
  if (!g || !out) return GBF_EINVAL;
  unsigned int* dmax = nullptr;
  GK(cudaMallocAsync((void**)&dmax, sizeof(unsigned int), g->stream));
  GK(cudaMemsetAsync(dmax, 0, sizeof(unsigned int), g->stream));
  max_kernel<<<blocks_for(g, 6 * g->d.nnode), kThreads, 0, g->stream>>>(g->ID, 6 * g->d.nnode, dmax);
  GK(cudaGetLastError());
  GK(cudaMemcpyAsync(out, dmax, sizeof(unsigned int), cudaMemcpyDeviceToHost, g->stream));
  GK(cudaFreeAsync(dmax, g->stream));
  GK(cudaStreamSynchronize(g->stream));
  return GBF_OK;
}

}  // extern "C"
