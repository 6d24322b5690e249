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

// Nodal indicator of a ball summed over its 3^d periodic images (GaNi
// topology): node x counts the images im in {-1,0,1}^d with
// sqrt(sum_a ((x_a - x0_a) - Y_a im_a)^2) < radius, each difference, square
// and sum rounded on its own as NumPy evaluates the reference's expression.
__global__ void __launch_bounds__(kInvThreads)
    k_ball_topology(const double* __restrict__ ax0, const double* __restrict__ ax1,
                    const double* __restrict__ ax2, int dim, int n0, int n1, int n2, double x00,
                    double x01, double x02, double Y0, double Y1, double Y2, double radius,
                    double* __restrict__ out) {
  const int i0 = blockIdx.z, i1 = blockIdx.y;
  const long long row = ((long long)i0 * n1 + i1) * n2;
  const double u0 = dim == 3 ? __dsub_rn(ax0[i0], x00) : 0.;
  const double u1 = __dsub_rn(ax1[i1], x01);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x) {
    const double u2 = __dsub_rn(ax2[j], x02);
    double cnt = 0.;
    for (int m0 = (dim == 3 ? -1 : 0); m0 <= (dim == 3 ? 1 : 0); ++m0)
      for (int m1 = -1; m1 <= 1; ++m1)
        for (int m2 = -1; m2 <= 1; ++m2) {
          double r2 = 0.;
          if (dim == 3) {
            const double a = __dsub_rn(u0, Y0 * m0);
            r2 = __dmul_rn(a, a);
          }
          const double b = __dsub_rn(u1, Y1 * m1);
          r2 = __dadd_rn(r2, __dmul_rn(b, b));
          const double c = __dsub_rn(u2, Y2 * m2);
          r2 = __dadd_rn(r2, __dmul_rn(c, c));
          if (__dsqrt_rn(r2) < radius) cnt += 1.;
        }
    out[row + j] = cnt;
  }
}

// Half spectrum (FFT order, [n0][n1][n2/2+1]) of the Hermitian part of
// X = W(|xi|) prod_a ph_a, the exact-integration spectrum of a ball
// inclusion: W = r^2 J1(2 pi r rho) / (r rho) / |Y| with rho^2 = sum_a sq_a
// (pi r^2 / |Y| at xi = 0), ph_a the per-axis phases.  Tables are indexed by
// the centred position i_a = (k_a + n_a/2) mod n_a of frequency k_a; -k_a sits
// at (n_a/2 - k_a) mod n_a with the same sq.  The real part of the full
// inverse transform of X is the c2r transform of (X(k) + conj X(-k)) / 2.
__global__ void __launch_bounds__(kInvThreads)
    k_ball_spectrum(const double* __restrict__ sq, const double2* __restrict__ ph, int n0,
                    int n1, int n2, double r, double inv_vol, double2* __restrict__ S) {
  const int n2h = n2 / 2 + 1;
  const int k0 = blockIdx.z, k1 = blockIdx.y;
  const int c0 = n0 / 2, c1 = n1 / 2, c2 = n2 / 2;
  const int i0 = (k0 + c0) % n0, m0 = (n0 - k0 + c0) % n0;
  const int i1 = (k1 + c1) % n1, m1 = (n1 - k1 + c1) % n1;
  const double* sq0 = sq;
  const double* sq1 = sq + n0;
  const double* sq2 = sq + n0 + n1;
  const double2* ph0 = ph;
  const double2* ph1 = ph + n0;
  const double2* ph2 = ph + n0 + n1;
  const double2 pa = ph0[i0], pb = ph0[m0];
  const double2 qa = ph1[i1], qb = ph1[m1];
  // ((1 ph0) ph1): the outer product in axis order
  const double2 ea = make_double2(pa.x * qa.x - pa.y * qa.y, pa.x * qa.y + pa.y * qa.x);
  const double2 eb = make_double2(pb.x * qb.x - pb.y * qb.y, pb.x * qb.y + pb.y * qb.x);
  const double s01 = __dadd_rn(sq0[i0], sq1[i1]);
  const long long row = ((long long)k0 * n1 + k1) * n2h;
  for (int k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 < n2h; k2 += gridDim.x * blockDim.x) {
    const int i2 = (k2 + c2) % n2, m2 = (n2 - k2 + c2) % n2;
    double w;
    if (i0 == c0 && i1 == c1 && i2 == c2) {
      w = M_PI * r * r * inv_vol;
    } else {
      const double rho = sqrt(__dadd_rn(s01, sq2[i2]));
      w = (r * r * j1(2. * M_PI * rho * r)) / (rho * r) * inv_vol;
    }
    const double2 fa = ph2[i2], fb = ph2[m2];
    const double2 xa = make_double2(ea.x * fa.x - ea.y * fa.y, ea.x * fa.y + ea.y * fa.x);
    const double2 xb = make_double2(eb.x * fb.x - eb.y * fb.y, eb.x * fb.y + eb.y * fb.x);
    S[row + k2] = make_double2(0.5 * w * (xa.x + xb.x), 0.5 * w * (xa.y - xb.y));
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

namespace fhp {

int ball_spectrum(const double* sq, const double* phase, int n0, int n1, int n2, double r,
                  double inv_vol, void* spec, void* stream) {
  const int n2h = n2 / 2 + 1;
  const int gx = (n2h + kInvThreads - 1) / kInvThreads;
  k_ball_spectrum<<<dim3(gx, n1, n0), kInvThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      sq, reinterpret_cast<const double2*>(phase), n0, n1, n2, r, inv_vol,
      static_cast<double2*>(spec));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(FHP_CUDA, std::string("k_ball_spectrum launch: ") + cudaGetErrorString(e));
  return FHP_OK;
}

}  // namespace fhp

extern "C" int fhp_ball_topology(int dim, const int* n, const double* axes, const double* x0,
                                 const double* Y, double radius, double* out, void* stream) {
  if (dim != 2 && dim != 3) return fail(FHP_BAD_ARG, "dim must be 2 or 3");
  if (!n || !axes || !x0 || !Y || !out) return fail(FHP_BAD_ARG, "n, axes, x0, Y and out are required");
  int g[3] = {1, 1, 1};
  int tot = 0;
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1 || n[i] > kInvMaxAxis)
      return fail(FHP_BAD_ARG, "grid size per axis must be between 1 and 65535");
    g[3 - dim + i] = n[i];
    tot += n[i];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* dax = nullptr;
  cudaError_t e = cudaMallocAsync(&dax, tot * sizeof(double), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dax, axes, tot * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    if (dax) cudaFreeAsync(dax, s);
    return fail(e == cudaErrorMemoryAllocation ? FHP_OOM : FHP_CUDA,
                std::string("ball topology set-up: ") + cudaGetErrorString(e));
  }
  // per-axis coordinate tables in the padded 3-axis order (axis 0 unused in 2D)
  const double* a0 = dax;
  const double* a1 = dim == 3 ? dax + n[0] : dax;
  const double* a2 = dim == 3 ? dax + n[0] + n[1] : dax + n[0];
  const double x00 = dim == 3 ? x0[0] : 0., Y0 = dim == 3 ? Y[0] : 0.;
  const int gx = (g[2] + kInvThreads - 1) / kInvThreads;
  k_ball_topology<<<dim3(gx, g[1], g[0]), kInvThreads, 0, s>>>(
      a0, a1, a2, dim, g[0], g[1], g[2], x00, x0[dim - 2], x0[dim - 1], Y0, Y[dim - 2],
      Y[dim - 1], radius, out);
  e = cudaGetLastError();
  cudaFreeAsync(dax, s);
  if (e != cudaSuccess)
    return fail(FHP_CUDA, std::string("k_ball_topology launch: ") + cudaGetErrorString(e));
  return FHP_OK;
}

namespace {

// One inclusion's values, passed by value (288 bytes of kernel parameters).
struct OuterValues { double v[36]; };

// out[k][i] += v[k] * c[i] for k < nv: the product and the sum rounded on
// their own, as NumPy's val += np.multiply.outer(v, c) rounds them.
__global__ void __launch_bounds__(256)
    k_outer_accumulate(const double* __restrict__ c, double* __restrict__ out, int nv,
                       const __grid_constant__ OuterValues vals, long long M) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += stride) {
    const double ci = c[i];
    for (int k = 0; k < nv; ++k) {
      double* o = out + (long long)k * M + i;
      *o = __dadd_rn(*o, __dmul_rn(vals.v[k], ci));
    }
  }
}

}  // namespace

extern "C" int fhp_outer_accumulate(int nv, const double* v, const double* c, double* out,
                                    long long M, void* stream) {
  if (nv < 1 || nv > 36) return fail(FHP_BAD_ARG, "nv must be between 1 and 36");
  if (!v || !c || !out || M < 1) return fail(FHP_BAD_ARG, "v, c, out and M >= 1 are required");
  const unsigned long long ob = (unsigned long long)nv * M * sizeof(double);
  const uintptr_t c0 = (uintptr_t)c, o0 = (uintptr_t)out;
  if (c0 < o0 + ob && o0 < c0 + (unsigned long long)M * sizeof(double))
    return fail(FHP_BAD_ARG, "c and out overlap");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  OuterValues vals{};
  for (int k = 0; k < nv; ++k) vals.v[k] = v[k];
  int nsm = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long need = (M + 255) / 256;
  const int grid = (int)(need < 8LL * nsm ? need : 8LL * nsm);
  k_outer_accumulate<<<grid, 256, 0, s>>>(c, out, nv, vals, M);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(FHP_CUDA, std::string("k_outer_accumulate launch: ") + cudaGetErrorString(e));
  return FHP_OK;
}

namespace {

// Separable characteristic functions: out[x] = prod_a t_a[x_a] (real tables)
// or the real part of prod_a c_a[x_a] (complex tables), in the order and
// with the roundings of NumPy's outer products: ((t0 t1) t2) for real tables;
// for complex ones c01 = c0 c1 with re = r0 r1 - i0 i1, im = r0 i1 + i0 r1,
// then re(c01 c2) = re01 r2 - im01 i2 (and re(c0 c1) for two axes).  Every
// product and difference rounded on its own.
__global__ void __launch_bounds__(256)
    k_separable_char(int dim, int n0, int n1, int n2, const double* __restrict__ re,
                     const double* __restrict__ im, double* __restrict__ out) {
  const long long M = (long long)n0 * n1 * n2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < M; v += stride) {
    const int i2 = (int)(v % n2);
    const long long r = v / n2;
    const int i1 = (int)(r % n1), i0 = (int)(r / n1);
    // tables are concatenated over the dim axes; 2D grids use (n1, n2)
    const int o1 = dim == 3 ? n0 : 0, o2 = o1 + n1;
    double t;
    if (!im) {
      t = dim == 3 ? __dmul_rn(__dmul_rn(re[i0], re[o1 + i1]), re[o2 + i2])
                   : __dmul_rn(re[o1 + i1], re[o2 + i2]);
    } else if (dim == 3) {
      const double r0 = re[i0], m0 = im[i0], r1 = re[o1 + i1], m1 = im[o1 + i1];
      const double cr = __dsub_rn(__dmul_rn(r0, r1), __dmul_rn(m0, m1));
      const double ci = __dadd_rn(__dmul_rn(r0, m1), __dmul_rn(m0, r1));
      t = __dsub_rn(__dmul_rn(cr, re[o2 + i2]), __dmul_rn(ci, im[o2 + i2]));
    } else {
      t = __dsub_rn(__dmul_rn(re[o1 + i1], re[o2 + i2]), __dmul_rn(im[o1 + i1], im[o2 + i2]));
    }
    out[v] = t;
  }
}

}  // namespace

extern "C" int fhp_separable_char(int dim, const int* n, const double* re, const double* im,
                                  double* out, void* stream) {
  if (dim != 2 && dim != 3) return fail(FHP_BAD_ARG, "dim must be 2 or 3");
  if (!n || !re || !out) return fail(FHP_BAD_ARG, "n, re and out are required");
  int tot = 0;
  for (int a = 0; a < dim; ++a) {
    if (n[a] < 1) return fail(FHP_BAD_ARG, "grid sizes must be positive");
    tot += n[a];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, (size_t)(im ? 2 : 1) * tot * sizeof(double), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d, re, tot * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && im)
    e = cudaMemcpyAsync(d + tot, im, tot * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    if (d) cudaFreeAsync(d, s);
    return fail(e == cudaErrorMemoryAllocation ? FHP_OOM : FHP_CUDA,
                std::string("separable tables: ") + cudaGetErrorString(e));
  }
  const int n0 = dim == 3 ? n[0] : 1, n1 = n[dim - 2], n2 = n[dim - 1];
  const long long M = (long long)n0 * n1 * n2;
  int nsm = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long need = (M + 255) / 256;
  const int grid = (int)(need < 8LL * nsm ? need : 8LL * nsm);
  k_separable_char<<<grid, 256, 0, s>>>(dim, n0, n1, n2, d, im ? d + tot : nullptr, out);
  e = cudaGetLastError();
  cudaFreeAsync(d, s);
  // the host tables are pageable: the copies have read them when the call
  // returns, the kernel runs in stream order
  if (e != cudaSuccess)
    return fail(FHP_CUDA, std::string("k_separable_char launch: ") + cudaGetErrorString(e));
  return FHP_OK;
}
