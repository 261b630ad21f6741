// fractal.cu — fractal fields on the device for #fractal_box and #add_surface_roughness
// (gprMax/fractals.py:141-194 and :29-111, filter fractals_generate_ext.pyx:24-86).
//
// The field is the real part of the inverse FFT of (FFT of seeded Gaussian noise) divided by
// r^D, with r the weighted distance of each frequency from the spectrum's centre. The noise is
// the caller's (the reference draws it with numpy's seeded generator); the transforms run in
// double precision with cuFFT, the filter and the final cast in kernels of this file. The
// reference evaluates fftshift(A) / B and then ifftshift; here the unshifted spectrum at index q
// is divided by B at the shifted index (q + n/2) mod n along each axis, which is the same
// quotient. The transforms round differently from the reference's FFT library, so the field
// agrees to rounding, not bit for bit.
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>
#include <cufft.h>

#include "../../include/gbfdtd.h"

namespace {

__global__ void to_complex(const double* __restrict__ x, cufftDoubleComplex* __restrict__ a, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    a[q] = make_cuDoubleComplex(x[q], 0.0);
}

struct FilterDims {
  int rank;
  int n[3];
  double w[3], v1[3];
  double D;
};

// A[q] /= B at the shifted index: B = (sum_a (w_a s_a - v1_a)^2)^(1/2)^D, 0.9 where it is 0;
// the DC term (index 0 of the unshifted array) is zeroed afterwards.
__global__ void filter(cufftDoubleComplex* __restrict__ a, long long n, const FilterDims f) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    long long r = q;
    double s2 = 0.0;
    for (int ax = f.rank - 1; ax >= 0; --ax) {
      const int idx = (int)(r % f.n[ax]);
      r /= f.n[ax];
      const int sh = (idx + f.n[ax] / 2) % f.n[ax];
      const double d = f.w[ax] * (double)sh - f.v1[ax];
      s2 += d * d;
    }
    const double rr = sqrt(s2);
    double B = pow(rr, f.D);
    if (B == 0.0) B = 0.9;
    cufftDoubleComplex v = a[q];
    v.x = v.x / B;
    v.y = v.y / B;
    if (q == 0) v = make_cuDoubleComplex(0.0, 0.0);
    a[q] = v;
  }
}

__global__ void real_part(const cufftDoubleComplex* __restrict__ a, float* __restrict__ out,
                          long long n, double scale) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    out[q] = (float)(a[q].x * scale);
}

}  // namespace

extern "C" int gbf_fractal_field(int32_t rank, const int32_t* dims, const double* weights,
                                 float dimension, const double* noise, float* field) {
  if ((rank != 2 && rank != 3) || !dims || !weights || !noise || !field) return GBF_EINVAL;
  long long n = 1;
  FilterDims f{};
  f.rank = rank;
  for (int a = 0; a < rank; ++a) {
    if (dims[a] < 1) return GBF_EINVAL;
    f.n[a] = dims[a];
    f.w[a] = weights[a];
    f.v1[a] = weights[a] * dims[a] / 2.0;
    n *= dims[a];
  }
  if (n > (1LL << 31)) return GBF_EINVAL;
  // D as the reference's compiled filter takes it: a float argument
  f.D = (double)dimension;
  double* x = nullptr;
  cufftDoubleComplex* a = nullptr;
  float* out = nullptr;
  cufftHandle plan = 0;
  bool planned = false;
  int rc = GBF_OK;
  cudaStream_t st = nullptr;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == GBF_OK) rc = e == cudaErrorMemoryAllocation ? GBF_ENOMEM : GBF_ECUDA;
    return rc == GBF_OK;
  };
  if (ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) &&
      ok(cudaMalloc((void**)&x, sizeof(double) * n)) &&
      ok(cudaMalloc((void**)&a, sizeof(cufftDoubleComplex) * n)) &&
      ok(cudaMalloc((void**)&out, sizeof(float) * n)) &&
      ok(cudaMemcpyAsync(x, noise, sizeof(double) * n, cudaMemcpyHostToDevice, st))) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8;
    to_complex<<<blocks, 256, 0, st>>>(x, a, n);
    cufftResult fr = rank == 3 ? cufftPlan3d(&plan, dims[0], dims[1], dims[2], CUFFT_Z2Z)
                               : cufftPlan2d(&plan, dims[0], dims[1], CUFFT_Z2Z);
    planned = fr == CUFFT_SUCCESS;
    if (planned) fr = cufftSetStream(plan, st);
    if (fr == CUFFT_SUCCESS) fr = cufftExecZ2Z(plan, a, a, CUFFT_FORWARD);
    if (fr == CUFFT_SUCCESS) {
      filter<<<blocks, 256, 0, st>>>(a, n, f);
      fr = cufftExecZ2Z(plan, a, a, CUFFT_INVERSE);
    }
    if (fr != CUFFT_SUCCESS) {
      rc = fr == CUFFT_ALLOC_FAILED ? GBF_ENOMEM : GBF_ECUDA;
    } else {
      // cuFFT's inverse is unnormalised; the reference's divides by the number of points
      real_part<<<blocks, 256, 0, st>>>(a, out, n, 1.0 / (double)n);
      if (ok(cudaGetLastError()))
        ok(cudaMemcpyAsync(field, out, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
      ok(cudaStreamSynchronize(st));
    }
  }
  if (planned) cufftDestroy(plan);
  if (st) cudaStreamSynchronize(st);
  cudaFree(x);
  cudaFree(a);
  cudaFree(out);
  if (st) cudaStreamDestroy(st);
  return rc;
}
