// fhp_coefficient_inverse: the dual coefficient A(x)^-1 of a field of d x d
// matrices, one thread per voxel, by Gauss-Jordan elimination without
// pivoting in the order of ffthompy/trigpol.py:120-159, optionally written
// with the grid ifftshift-ed (the centred-to-0 origin move of
// Material.get_A_GaNi, ffthompy/materials.py:115-123).
//
// The kernel reads d*d doubles and writes d*d doubles per voxel (the
// algorithmic traffic); the elimination costs about 2 d^3 FP64 operations and
// d (d+1) + d (d-1) / 2 divisions per voxel, which on GB300's FP64 rate is of
// the same order as the memory time at d = 6.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/ffthompy_gb300.h"
#include "fhp_engine.h"

namespace {

constexpr int kInvThreads = 128;
constexpr int kInvMaxD = 6;
constexpr int kInvMaxAxis = 65535;  // grid y / z limit: one block row per (n0, n1)

// Row m is divided by its pivot, then eliminated from the rows below it; the
// back substitution runs from the last row up.  Every product and every
// difference is rounded on its own (__dmul_rn / __dsub_rn never contract into
// a fused multiply-add) and divisions are IEEE, as NumPy evaluates the
// reference's array expressions, so results are bit-identical to it for
// finite input; a zero pivot gives the same Inf / NaN pattern.
template <int D>
__device__ __forceinline__ void gauss_jordan(double (&B)[D][D], double (&X)[D][D]) {
#pragma unroll
  for (int m = 0; m < D; ++m)
#pragma unroll
    for (int n = 0; n < D; ++n) X[m][n] = m == n ? 1. : 0.;
#pragma unroll
  for (int m = 0; m < D; ++m) {
    const double piv = B[m][m];
    B[m][m] = 1.;
#pragma unroll
    for (int n = m + 1; n < D; ++n) B[m][n] = __ddiv_rn(B[m][n], piv);
#pragma unroll
    for (int n = 0; n < D; ++n) X[m][n] = __ddiv_rn(X[m][n], piv);
#pragma unroll
    for (int k = m + 1; k < D; ++k) {
      const double f = B[k][m];
#pragma unroll
      for (int l = 0; l < D; ++l) {
        B[k][l] = __dsub_rn(B[k][l], __dmul_rn(B[m][l], f));
        X[k][l] = __dsub_rn(X[k][l], __dmul_rn(X[m][l], f));
      }
    }
  }
#pragma unroll
  for (int m = D - 1; m >= 0; --m)
#pragma unroll
    for (int k = m - 1; k >= 0; --k) {
      const double f = B[k][m];
#pragma unroll
      for (int l = 0; l < D; ++l) {
        B[k][l] = __dsub_rn(B[k][l], __dmul_rn(B[m][l], f));
        X[k][l] = __dsub_rn(X[k][l], __dmul_rn(X[m][l], f));
      }
    }
}

// Block (x, i1, i0) covers output row (i0, i1) of the last axis.  With shift,
// output voxel j takes input voxel (j + n/2) mod n on every axis (ifftshift).
template <int D>
__global__ void __launch_bounds__(kInvThreads)
    k_coef_inverse(const double* __restrict__ A, double* __restrict__ Ainv, int n0, int n1,
                   int n2, int shift) {
  const long long M = (long long)n0 * n1 * n2;
  const int i0 = blockIdx.z, i1 = blockIdx.y;
  int s0 = i0, s1 = i1, h2 = 0;
  if (shift) {
    s0 += n0 / 2;
    if (s0 >= n0) s0 -= n0;
    s1 += n1 / 2;
    if (s1 >= n1) s1 -= n1;
    h2 = n2 / 2;
  }
  const long long orow = ((long long)i0 * n1 + i1) * n2;
  const long long srow = ((long long)s0 * n1 + s1) * n2;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x) {
    int s2 = j + h2;
    if (s2 >= n2) s2 -= n2;
    double B[D][D], X[D][D];
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) B[m][n] = A[(long long)(m * D + n) * M + srow + s2];
    gauss_jordan<D>(B, X);
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) Ainv[(long long)(m * D + n) * M + orow + j] = X[m][n];
  }
}

int fail(int status, const std::string& msg) {
  fhp::set_error(msg);
  return status;
}

template <int D>
void launch(const double* A, double* Ainv, int n0, int n1, int n2, int shift, cudaStream_t s) {
  const int gx = (n2 + kInvThreads - 1) / kInvThreads;
  k_coef_inverse<D><<<dim3(gx, n1, n0), kInvThreads, 0, s>>>(A, Ainv, n0, n1, n2, shift);
}

}  // namespace

extern "C" int fhp_coefficient_inverse(int dim, const int* n, int d, const double* A,
                                       double* Ainv, int shift, void* stream) {
  if (dim < 1 || dim > 3) return fail(FHP_BAD_ARG, "dim must be 1, 2 or 3");
  if (!n || !A || !Ainv) return fail(FHP_BAD_ARG, "n, A and Ainv are required");
  if (d < 1 || d > kInvMaxD) return fail(FHP_BAD_ARG, "d must be between 1 and 6");
  int g[3] = {1, 1, 1};
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1 || n[i] > kInvMaxAxis)
      return fail(FHP_BAD_ARG, "grid size per axis must be between 1 and 65535");
    g[3 - dim + i] = n[i];
  }
  const unsigned long long bytes =
      (unsigned long long)d * d * g[0] * g[1] * g[2] * sizeof(double);
  const uintptr_t a0 = (uintptr_t)A, b0 = (uintptr_t)Ainv;
  if (a0 < b0 + bytes && b0 < a0 + bytes) return fail(FHP_BAD_ARG, "A and Ainv overlap");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (d) {
    case 1: launch<1>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
    case 2: launch<2>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
    case 3: launch<3>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
    case 4: launch<4>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
    case 5: launch<5>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
    default: launch<6>(A, Ainv, g[0], g[1], g[2], shift != 0, s); break;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(FHP_CUDA, std::string("k_coef_inverse launch: ") + cudaGetErrorString(e));
  return FHP_OK;
}
