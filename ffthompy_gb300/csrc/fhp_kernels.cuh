// Kernels of the Fourier-Galerkin operator G o A, CG and postprocessing.
//
// Layouts (C order, all on one GPU):
//   real field   x[comp][n0][n1][n2],  comp = load*dv + c, M = n0*n1*n2 voxels
//   spectrum     S[comp][n0][n1][n2h], n2h = n2/2+1 (numpy rfftn half spectrum)
//   coefficient  A[a][n0][n1][n2]: 1 (isotropic a*I), dv*(dv+1)/2 (symmetric,
//                packed upper triangle) or dv*dv (full) values per voxel
// 2D grids use n0 = 1.  The operator is FiGFA = iF o G o F o A
// (ffthompy/applications.py:58 with Operator's reversed factor order,
// ffthompy/tensors/operators.py:119-144).
#pragma once
#include <cuda.h>   // CUtensorMap (a kernel parameter type; no driver call here)

#include "fhp_fft.cuh"

namespace fhp {

enum CoefKind { COEF_NONE = 0, COEF_ISO = 1, COEF_SYM = 2, COEF_FULL = 3 };

struct LoadState {
  double rr;        // <R,R>
  double pap;       // <P,AP>
  double alpha;
  double beta;
  double norm_res;  // sqrt(rr)
  double tol;
  int kit;
  int maxiter;
  int done;
  int status;       // 0 ok, 1 stagnated (FP32), 2 breakdown (p.Ap <= 0), 3 non-finite
  double min_norm;  // smallest residual norm so far
  double guard;     // stop when norm_res > guard * min_norm (0: off)
};

struct GridDims {
  int dim;        // 2 or 3
  int n0, n1, n2; // n0 = 1 for 2D
  int n2h;
  int dv;         // components per load
  int L;          // loads
  long long M;    // voxels
  FastDiv dn2, dn2h, dnp;  // division by n2, n2h and the pair-line count (L*dv+1)/2
  // a plan batched over K cells of the same grid: cell k's fields, spectra and
  // coefficient start k * sf, k * ss, k * sa elements further, its loads'
  // states k * L entries further; the passes take the cell from the grid's
  // instance dimension (K = 1: one cell)
  int K = 1;
  long long sf = 0, ss = 0, sa = 0;
};

inline void set_grid_divs(GridDims& g) {
  g.dn2 = make_fastdiv((unsigned)g.n2);
  g.dn2h = make_fastdiv((unsigned)g.n2h);
  g.dnp = make_fastdiv((unsigned)((g.L * g.dv + 1) / 2));
}

// FFT pass kernels: two CTAs per SM (128 registers) for FP32; FP64 values take
// two registers each, so the FP64 instantiations keep one CTA per SM and the
// full register file instead of spilling.
template <typename R> constexpr int kFftMinBlocks = sizeof(R) == 4 ? 2 : 1;

constexpr int kMaxDv = 6;
constexpr int kMaxLoads = 6;

// Green projection parameters (ffthompy/projections.py:9-267)
struct GreenParams {
  int physics;    // 0 scalar, 1 elasticity (Mandel)
  int proj;       // 1: G1 (compatible, primal), 2: G2 (equilibrated, dual), 0: band only
  int h[3];       // band half-widths |k_i| <= h_i, real axis order
  double Y[3];    // cell size, real axis order
  double invY[3]; // 1 / Y
  double scale;   // Ga scale prod(2N-1)/prod(N); 1 for GaNi
};

__device__ __forceinline__ int signed_freq(int k, int n) { return (2 * k <= n) ? k : k - n; }

// Mandel index -> tensor pair and weight (3D order 0..5: 00 11 22 12 02 01;
// 2D order 0..2: 00 11 01), ffthompy/projections.py:196-229.
__device__ __forceinline__ void mandel_pair(int dim, int I, int& a, int& b) {
  if (dim == 3) {
    const int aa[6] = {0, 1, 2, 1, 0, 0};
    const int bb[6] = {0, 1, 2, 2, 2, 1};
    a = aa[I]; b = bb[I];
  } else {
    const int aa[3] = {0, 1, 0};
    const int bb[3] = {0, 1, 1};
    a = aa[I]; b = bb[I];
  }
}

// y = G(xi) x for one frequency, G from the closed forms:
//   scalar:     G1 = xi xi^T / |xi|^2,           G2 = I - G1
//   elasticity: G1 e = sym(n (x) e n)*2 - n n (n.e.n), Mandel-weighted, G2 = I - G1
// zero at k = 0 and outside the band; times scale.  DIM is a template
// parameter so every small array is indexed by constants (registers).
template <typename R, int DIM, int PHYS>
__device__ __forceinline__ void green_apply_d(const GreenParams& gp, const int* k,
                                              cplx<R>* x /* in/out, dv values */) {
  constexpr int DVE = PHYS == 0 ? DIM : DIM * (DIM + 1) / 2;
  bool inband = true, zero = true;
  R xi[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    const int ki = k[i];
    if (ki > gp.h[i] || -ki > gp.h[i]) inband = false;
    if (ki != 0) zero = false;
    xi[i] = R(ki) * R(gp.invY[i]);
  }
  constexpr bool scalar = PHYS == 0;
  const R s = R(gp.scale);
  if (gp.proj == 0) {  // no projection (energies): scale only
#pragma unroll
    for (int c = 0; c < DVE; ++c)
      if (!scalar || c < DIM) x[c] = cscale<R>(x[c], s);
    return;
  }
  if (!inband || zero) {
#pragma unroll
    for (int c = 0; c < DVE; ++c)
      if (!scalar || c < DIM) x[c] = mkc<R>(R(0), R(0));
    return;
  }
  R nn = R(0);
#pragma unroll
  for (int i = 0; i < DIM; ++i) nn += xi[i] * xi[i];
  if constexpr (scalar) {
    // (xi . x) / |xi|^2
    cplx<R> t = mkc<R>(R(0), R(0));
#pragma unroll
    for (int i = 0; i < DIM; ++i) { t.x += xi[i] * x[i].x; t.y += xi[i] * x[i].y; }
    const R inn = R(1) / nn;
    t.x *= inn;
    t.y *= inn;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      cplx<R> g1 = mkc<R>(xi[i] * t.x, xi[i] * t.y);
      x[i] = (gp.proj == 1) ? cscale<R>(g1, s) : cscale<R>(csub<R>(x[i], g1), s);
    }
    return;
  } else {
  // elasticity: unit normal, strain tensor from Mandel vector
  const R inv = R(1) / sqrt(nn);
  R n[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) n[i] = xi[i] * inv;
  const R isq2 = R(0.70710678118654752440084436210485);
  cplx<R> e[DIM][DIM];
#pragma unroll
  for (int I = 0; I < DVE; ++I) {
    int a, b;
    mandel_pair(DIM, I, a, b);
    if (a == b) e[a][a] = x[I];
    else { e[a][b] = cscale<R>(x[I], isq2); e[b][a] = e[a][b]; }
  }
  cplx<R> en[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    en[i] = mkc<R>(R(0), R(0));
#pragma unroll
    for (int j = 0; j < DIM; ++j) { en[i].x += e[i][j].x * n[j]; en[i].y += e[i][j].y * n[j]; }
  }
  cplx<R> nen = mkc<R>(R(0), R(0));
#pragma unroll
  for (int i = 0; i < DIM; ++i) { nen.x += n[i] * en[i].x; nen.y += n[i] * en[i].y; }
  const R sq2 = R(1.4142135623730950488016887242097);
#pragma unroll
  for (int I = 0; I < DVE; ++I) {
    int a, b;
    mandel_pair(DIM, I, a, b);
    // (G1 e)_ab = n_a (e n)_b + n_b (e n)_a - n_a n_b (n.e.n)
    cplx<R> g = mkc<R>(n[a] * en[b].x + n[b] * en[a].x - n[a] * n[b] * nen.x,
                       n[a] * en[b].y + n[b] * en[a].y - n[a] * n[b] * nen.y);
    if (a != b) g = cscale<R>(g, sq2);
    x[I] = (gp.proj == 1) ? cscale<R>(g, s) : cscale<R>(csub<R>(x[I], g), s);
  }
  }
}

// PHYS is a template parameter of the kernels that call this, so a scalar
// plan's kernels carry no elasticity code (and its register demand).
template <typename R, int PHYS>
__device__ __forceinline__ void green_apply(const GreenParams& gp, int dim, const int* k,
                                            cplx<R>* x /* in/out, dv values */) {
  if (dim == 3) green_apply_d<R, 3, PHYS>(gp, k, x);
  else green_apply_d<R, 2, PHYS>(gp, k, x);
}

// q = A(v) x for one voxel and one load; A component-major with stride M.
// Loops run to kMaxDv with a guard so x and q stay in registers.
template <typename R, int COEF>
__device__ __forceinline__ void coef_apply(const R* __restrict__ A, long long M, long long v,
                                           int dv, const R* x, R* q) {
  if constexpr (COEF == COEF_NONE) {
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < dv) q[c] = x[c];
  } else if constexpr (COEF == COEF_ISO) {
    const R a = A[v];
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < dv) q[c] = a * x[c];
  } else if constexpr (COEF == COEF_SYM) {
#pragma unroll
    for (int a = 0; a < kMaxDv; ++a) {
      if (a >= dv) break;
      R s = R(0);
#pragma unroll
      for (int b = 0; b < kMaxDv; ++b) {
        if (b >= dv) break;
        const int i = a < b ? a : b, j = a < b ? b : a;
        const int t = i * dv - i * (i - 1) / 2 + (j - i);
        s += A[(long long)t * M + v] * x[b];
      }
      q[a] = s;
    }
  } else {
#pragma unroll
    for (int a = 0; a < kMaxDv; ++a) {
      if (a >= dv) break;
      R s = R(0);
#pragma unroll
      for (int b = 0; b < kMaxDv; ++b) {
        if (b >= dv) break;
        s += A[(long long)(a * dv + b) * M + v] * x[b];
      }
      q[a] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// block reductions (double)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Reduces acc[0..n) over the block; threads i < n write out[i].  red must hold
// (blockDim/32)*n doubles.  The loop runs to the array size with a guard so
// acc stays in registers.
template <int NMAX>
__device__ __forceinline__ void block_sum_n(double (&acc)[NMAX], int n, double* red, double* out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NMAX; ++i) {
    if (i >= n) break;
    double v = warp_sum(acc[i]);
    if (lane == 0) red[w * n + i] = v;
  }
  __syncthreads();
  if (threadIdx.x < n) {
    double s = 0.;
    for (int j = 0; j < nw; ++j) s += red[j * n + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------
// pass 1: r2c along the last axis, with the coefficient multiply in the
// prologue and (CG) the direction update P = R + beta P.
// CTA: `rows` consecutive (i0,i1) rows, all comps; comps paired as z = a + i b.
// every load of a cell has stopped (the CG passes skip the cell)
__device__ __forceinline__ bool cell_done(const LoadState* __restrict__ st, int L) {
  for (int l = 0; l < L; ++l)
    if (!st[l].done) return false;
  return true;
}

// ---------------------------------------------------------------------------
template <typename R, int COEF, bool PUPD>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_r2c_last(
    const R* __restrict__ xin, R* __restrict__ pio, const R* __restrict__ rvec,
    const R* __restrict__ A, cplx<R>* __restrict__ S, const __grid_constant__ GridDims g, const __grid_constant__ LineDev<R> L, int rows,
    const LoadState* __restrict__ st, const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  {  // the cell of a batched plan (grid y)
    const long long k = blockIdx.y;
    if (xin) xin += k * g.sf;
    if (pio) pio += k * g.sf;
    if (rvec) rvec += k * g.sf;
    if (A) A += k * g.sa;
    S += k * g.ss;
    if (st) st += k * g.L;
  }
  if (all_done && st && cell_done(st, g.L)) return;   // CG only (all_done given)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int C = g.L * g.dv;
  const int np = (C + 1) / 2;
  const int ld = L.ld;
  const long long nrows = (long long)g.n0 * g.n1;
  const long long row0 = (long long)blockIdx.x * rows;
  const int n = g.n2;
  const int tasks = rows * n;
  // per-load beta and activity, read once (not per voxel)
  R betl[kMaxLoads];
  bool wrl[kMaxLoads];
#pragma unroll
  for (int l = 0; l < kMaxLoads; ++l) {
    betl[l] = (PUPD && l < g.L) ? R(st[l].beta) : R(0);
    wrl[l] = PUPD && l < g.L && !st[l].done;
  }
  for (int e = threadIdx.x; e < tasks; e += blockDim.x) {
    const int rl = fdiv(e, g.dn2), j = e - rl * n;
    const long long row = row0 + rl;
    cplx<R>* base = buf + (long long)rl * np * ld;
    if (row >= nrows) {
      for (int p = 0; p < np; ++p) base[p * ld + sp(j)] = mkc<R>(R(0), R(0));
      continue;
    }
    const long long v = row * n + j;
#pragma unroll
    for (int l = 0; l < kMaxLoads; ++l) {
      if (l >= g.L) break;
      R xv[kMaxDv], q[kMaxDv], rv[kMaxDv];
      // every global load of this load case before any store
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const long long idx = (long long)(l * g.dv + c) * g.M + v;
        xv[c] = PUPD ? pio[idx] : xin[idx];
        if constexpr (PUPD) rv[c] = rvec[idx];
      }
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        if constexpr (PUPD) {
          const long long idx = (long long)(l * g.dv + c) * g.M + v;
          xv[c] = rv[c] + betl[l] * xv[c];
          if (wrl[l]) pio[idx] = xv[c];
        }
      }
      coef_apply<R, COEF>(A, g.M, v, g.dv, xv, q);
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const int comp = l * g.dv + c;
        cplx<R>* line = base + (comp >> 1) * ld;
        // slot j of the pair line: real part from even comp, imag from odd
        R* slot = reinterpret_cast<R*>(line + sp(j)) + (comp & 1);
        *slot = q[c];
      }
    }
    if (C & 1) reinterpret_cast<R*>(base + (np - 1) * ld + sp(j))[1] = R(0);
  }
  __syncthreads();
  if (L.blue) {
    // chirp pre-multiply of the stored values (put_fwd for Bluestein lines)
    for (int e = threadIdx.x; e < rows * np * n; e += blockDim.x) {
      const int line = fdiv(e, g.dn2), j = e - line * n;
      cplx<R>* p = buf + (long long)line * ld + sp(j);
      *p = cmul<R>(*p, L.chirp[j]);
    }
  }
  zero_tail<R>(buf, ld, rows * np, L);
  __syncthreads();
  line_core<R>(buf, ld, rows * np, L, false);
  // split the paired spectra: Xa = (Z_k + conj Z_{n-k})/2, Xb = (Z_k - conj Z_{n-k})/(2i)
  // (one warp per pair line, lanes over k: coalesced stores, no division per element)
  const int n2h = g.n2h;
  const int lane = threadIdx.x & 31;
  for (int line = threadIdx.x >> 5; line < rows * np; line += blockDim.x >> 5) {
    const int rl = fdiv(line, g.dnp), p = line - rl * np;
    const long long row = row0 + rl;
    if (row >= nrows) continue;
    const cplx<R>* lp = buf + (long long)line * ld;
    const int ca = 2 * p, cb = 2 * p + 1;
    cplx<R>* da = S + ((long long)ca * nrows + row) * n2h;
    cplx<R>* db = S + ((long long)cb * nrows + row) * n2h;
    for (int k = lane; k < n2h; k += 32) {
      const cplx<R> zk = get_fwd<R>(lp, L, k);
      const cplx<R> zm = get_fwd<R>(lp, L, k == 0 ? 0 : n - k);
      da[k] = mkc<R>(R(0.5) * (zk.x + zm.x), R(0.5) * (zk.y - zm.y));
      if (cb < C) db[k] = mkc<R>(R(0.5) * (zk.y + zm.y), R(0.5) * (zm.x - zk.x));
    }
  }
}

// ---------------------------------------------------------------------------
// strided c2c pass: lines of length na along an axis with `inner` contiguous
// elements after it; CTA = tile of T inner columns of one outer index.
// ---------------------------------------------------------------------------
template <typename R, bool INV>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_c2c_axis(cplx<R>* __restrict__ S, int na, long long inner,
                                                  const __grid_constant__ LineDev<R> L, int T,
                                                  const int* __restrict__ all_done,
                                                  const LoadState* __restrict__ st,
                                                  int outer_per_load, long long cell_stride,
                                                  int cell_loads) {
  if (all_done && *all_done) return;
  // the cell of a batched plan (grid z): spectra cell_stride further, states
  // cell_loads further
  S += (long long)blockIdx.z * cell_stride;
  if (st) st += (long long)blockIdx.z * cell_loads;
  if (st && outer_per_load > 0 && st[blockIdx.y / outer_per_load].done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int ld = L.ld;
  const long long t0 = (long long)blockIdx.x * T;
  cplx<R>* base = S + (long long)blockIdx.y * na * inner;
  const int tasks = T * na;
  const int lgT = __ffs(T) - 1;  // T is a power of two
  // copies go straight to their slots (many in flight per thread)
  for (int e = threadIdx.x; e < tasks; e += blockDim.x) {
    const int i = e >> lgT, t = e & (T - 1);
    const long long col = t0 + t;
    cplx<R>* slot = buf + t * ld + (INV ? slot_inv<R>(L, i) : slot_fwd<R>(L, i));
    if (col < inner) cp_async_cplx<R>(slot, base + (long long)i * inner + col);
    else *slot = mkc<R>(R(0), R(0));
  }
  cp_async_commit();
  zero_tail<R>(buf, ld, T, L);
  cp_async_wait<0>();
  __syncthreads();
  if (L.blue) {
    blue_fixup<R, INV>(buf, ld, T, L);
    __syncthreads();
  }
  line_core<R>(buf, ld, T, L, INV);
  for (int e = threadIdx.x; e < tasks; e += blockDim.x) {
    const int i = e >> lgT, t = e & (T - 1);
    const long long col = t0 + t;
    if (col >= inner) continue;
    base[(long long)i * inner + col] = INV ? get_inv<R>(buf + t * ld, L, i)
                                           : get_fwd<R>(buf + t * ld, L, i);
  }
}

// ---------------------------------------------------------------------------
// projection pass on the first real axis: forward line DFT, y = G(xi) x over
// the dv comps of each frequency, inverse line DFT.  CTA = T inner columns of
// one load; lines (c, t) for c < dv.
// ---------------------------------------------------------------------------
template <typename R, int PHYS>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_proj_first(cplx<R>* __restrict__ S, const __grid_constant__ GridDims g, int na,
                                                    long long inner, const __grid_constant__ LineDev<R> L, int T,
                                                    const __grid_constant__ GreenParams gp,
                                                    const int* __restrict__ all_done,
                                                    const LoadState* __restrict__ st) {
  if (all_done && *all_done) return;
  const int l = blockIdx.y;
  S += (long long)blockIdx.z * g.ss;          // the cell of a batched plan
  if (st) st += (long long)blockIdx.z * g.L;
  if (st && st[l].done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int ld = L.ld;
  const int dv = g.dv;
  const long long t0 = (long long)blockIdx.x * T;
  const int nl = dv * T;
  const int tasks = nl * na;
  const int lgT = __ffs(T) - 1;  // T is a power of two
  // coalesced load: consecutive threads take consecutive inner columns
  for (int e = threadIdx.x; e < tasks; e += blockDim.x) {
    const int t = e & (T - 1);
    const int rest = e >> lgT;
    const int c = fdiv(rest, L.dn);
    const int i = rest - c * na;
    const long long col = t0 + t;
    const cplx<R>* src = S + ((long long)(l * dv + c) * na) * inner;
    cplx<R>* slot = buf + (c * T + t) * ld + slot_fwd<R>(L, i);
    if (col < inner) cp_async_cplx<R>(slot, src + (long long)i * inner + col);
    else *slot = mkc<R>(R(0), R(0));
  }
  cp_async_commit();
  zero_tail<R>(buf, ld, nl, L);
  cp_async_wait<0>();
  __syncthreads();
  if (L.blue) {
    blue_fixup<R, false>(buf, ld, nl, L);
    __syncthreads();
  }
  line_core<R>(buf, ld, nl, L, false);
  // Green projection per frequency
  const int ftasks = T * na;
  for (int e = threadIdx.x; e < ftasks; e += blockDim.x) {
    const int t = e & (T - 1), k = e >> lgT;
    const long long col = t0 + t;
    cplx<R> x[kMaxDv];
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < dv) x[c] = get_fwd<R>(buf + (c * T + t) * ld, L, k);
    if (col < inner) {
      int kv[3];
      kv[0] = signed_freq(k, na);
      if (g.dim == 3) {
        const int k1 = fdiv((int)col, g.dn2h);
        kv[1] = signed_freq(k1, g.n1);
        kv[2] = (int)col - k1 * g.n2h;
      } else {
        kv[1] = (int)col;
        kv[2] = 0;
      }
      green_apply<R, PHYS>(gp, g.dim, kv, x);
    }
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < dv) put_inv<R>(buf + (c * T + t) * ld, L, k, x[c]);
  }
  __syncthreads();
  zero_tail<R>(buf, ld, nl, L);
  __syncthreads();
  line_core<R>(buf, ld, nl, L, true);
  for (int e = threadIdx.x; e < tasks; e += blockDim.x) {
    const int t = e & (T - 1);
    const int rest = e >> lgT;
    const int c = fdiv(rest, L.dn);
    const int i = rest - c * na;
    const long long col = t0 + t;
    if (col >= inner) continue;
    cplx<R>* dst = S + ((long long)(l * dv + c) * na) * inner;
    dst[(long long)i * inner + col] = get_inv<R>(buf + (c * T + t) * ld, L, i);
  }
}

// ---------------------------------------------------------------------------
// last pass: c2r along the last axis (pairs of comps), scale, store; optional
// fused dot <p, y> per load (CG's <P, AP>).
// ---------------------------------------------------------------------------
template <typename R, bool DOT>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_c2r_last(const cplx<R>* __restrict__ S, R* __restrict__ y,
                                                  const R* __restrict__ pdot,
                                                  double* __restrict__ partials, const __grid_constant__ GridDims g,
                                                  const __grid_constant__ LineDev<R> L, int rows, R scale,
                                                  const int* __restrict__ all_done, int stage,
                                                  const LoadState* __restrict__ st) {
  if (all_done && *all_done) return;
  {  // the cell of a batched plan (grid y); partial sums [cell][CTA][load]
    const long long k = blockIdx.y;
    S += k * g.ss;
    y += k * g.sf;
    if (pdot) pdot += k * g.sf;
    if (partials) partials += k * gridDim.x * g.L;
    if (st) st += k * g.L;
  }
  if (st && cell_done(st, g.L)) return;   // CG only: a cell whose loads have all stopped
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int C = g.L * g.dv;
  const int np = (C + 1) / 2;
  const int ld = L.ld;
  const long long nrows = (long long)g.n0 * g.n1;
  const long long row0 = (long long)blockIdx.x * rows;
  const int n = g.n2, n2h = g.n2h;
  // stage this CTA's spectra (C contiguous runs of vrows*n2h) when they fit
  const int vrows = (int)((nrows - row0) < rows ? (nrows - row0) : rows);
  cplx<R>* sraw = reinterpret_cast<cplx<R>*>(
      smem_raw + align16((size_t)rows * np * ld * sizeof(cplx<R>)));
  if (stage) {
    for (int c = 0; c < C; ++c)
      stage_async(sraw + (size_t)c * rows * n2h, S + ((long long)c * nrows + row0) * n2h,
                  vrows * n2h);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
  }
  // one warp per pair line, lanes over k (no division per element)
  for (int line = threadIdx.x >> 5; line < rows * np; line += blockDim.x >> 5) {
    const int rl = fdiv(line, g.dnp), p = line - rl * np;
    const long long row = row0 + rl;
    cplx<R>* lp = buf + (long long)line * ld;
    const int ca = 2 * p, cb = 2 * p + 1;
    const bool valid = row < nrows;
    const cplx<R>* sa = stage ? sraw + ((size_t)ca * rows + rl) * n2h
                              : S + ((long long)ca * nrows + row) * n2h;
    const cplx<R>* sb = stage ? sraw + ((size_t)cb * rows + rl) * n2h
                              : S + ((long long)cb * nrows + row) * n2h;
    for (int k = (int)(threadIdx.x & 31); k < n2h; k += 32) {
      cplx<R> a = mkc<R>(R(0), R(0)), b = mkc<R>(R(0), R(0));
      if (valid) {
        a = sa[k];
        if (cb < C) b = sb[k];
      }
      const bool selfconj = (k == 0) || (2 * k == n);
      if (selfconj) { a.y = R(0); b.y = R(0); }
      // Z_k = A + iB ; Z_{n-k} = conj(A) + i conj(B)
      put_inv<R>(lp, L, k, mkc<R>(a.x - b.y, a.y + b.x));
      if (!selfconj) put_inv<R>(lp, L, n - k, mkc<R>(a.x + b.y, b.x - a.y));
    }
  }
  zero_tail<R>(buf, ld, rows * np, L);
  __syncthreads();
  line_core<R>(buf, ld, rows * np, L, true);
  double acc[kMaxLoads];
#pragma unroll
  for (int i = 0; i < kMaxLoads; ++i) acc[i] = 0.;
  // one warp per pair line: the <p, y> terms of a line add up per lane in the
  // field precision (at most n/32 terms) and reach the FP64 accumulators once
  // per line (FP64 arithmetic per element would dominate on this part)
  const int lane = threadIdx.x & 31;
  for (int line = threadIdx.x >> 5; line < rows * np; line += blockDim.x >> 5) {
    const int rl = fdiv(line, g.dnp), p = line - rl * np;
    const long long row = row0 + rl;
    if (row >= nrows) continue;
    const cplx<R>* lp = buf + (long long)line * ld;
    const int ca = 2 * p, cb = 2 * p + 1;
    R* ya_out = y + (long long)ca * g.M + row * n;
    R* yb_out = y + (long long)cb * g.M + row * n;
    R sa = R(0), sb = R(0);
    // unrolled: the P loads of several j are in flight together
#pragma unroll 4
    for (int j = lane; j < n; j += 32) {
      const cplx<R> z = get_inv<R>(lp, L, j);
      const R ya = z.x * scale, yb = z.y * scale;
      ya_out[j] = ya;
      if (cb < C) yb_out[j] = yb;
      if constexpr (DOT) {
        sa += pdot[(long long)ca * g.M + row * n + j] * ya;
        if (cb < C) sb += pdot[(long long)cb * g.M + row * n + j] * yb;
      }
    }
    if constexpr (DOT) {
      const int la = ca / g.dv, lb = cb < C ? cb / g.dv : -1;
      // constant indices: acc stays in registers
#pragma unroll
      for (int l = 0; l < kMaxLoads; ++l) {
        if (l == la) acc[l] += (double)sa;
        if (l == lb) acc[l] += (double)sb;
      }
    }
  }
  if constexpr (DOT) {
    __syncthreads();
    double* red = reinterpret_cast<double*>(smem_raw);
    block_sum_n(acc, g.L, red, partials + (long long)blockIdx.x * g.L);
  }
}

// ---------------------------------------------------------------------------
// CG helpers
// ---------------------------------------------------------------------------
// partial sums of <x, y> per load (grid-stride over voxels)
template <typename R>
__global__ void __launch_bounds__(256) k_dot(const R* __restrict__ x, const R* __restrict__ y,
                                             double* __restrict__ partials, GridDims g) {
  x += (long long)blockIdx.y * g.sf;        // the cell of a batched plan (grid y)
  y += (long long)blockIdx.y * g.sf;
  partials += (long long)blockIdx.y * gridDim.x * g.L;
  __shared__ double red[8 * kMaxLoads];
  double acc[kMaxLoads];
  R part[kMaxLoads];   // up to 8 voxels per thread in the field precision
  for (int i = 0; i < kMaxLoads; ++i) {
    acc[i] = 0.;
    part[i] = R(0);
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  int cnt = 0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
#pragma unroll
    for (int l = 0; l < kMaxLoads; ++l) {
      if (l >= g.L) break;
      for (int c = 0; c < g.dv; ++c) {
        const long long i = (long long)(l * g.dv + c) * g.M + v;
        part[l] += x[i] * y[i];
      }
    }
    // into FP64 every 8 voxels: FP64 arithmetic is the slow pipe on this GPU
    if (++cnt == 8) {
#pragma unroll
      for (int l = 0; l < kMaxLoads; ++l) {
        acc[l] += (double)part[l];
        part[l] = R(0);
      }
      cnt = 0;
    }
  }
#pragma unroll
  for (int l = 0; l < kMaxLoads; ++l) acc[l] += (double)part[l];
  block_sum_n(acc, g.L, red, partials + (long long)blockIdx.x * g.L);
}

// x += alpha P ; R -= alpha AP ; partial <R,R>   (ffthompy/general/solver.py:127-129)
template <typename R>
__global__ void __launch_bounds__(256) k_cg_update(R* __restrict__ x, R* __restrict__ r,
                                                   const R* __restrict__ p,
                                                   const R* __restrict__ ap,
                                                   double* __restrict__ partials, GridDims g,
                                                   const LoadState* __restrict__ st,
                                                   const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8 * kMaxLoads];
  double acc[kMaxLoads];
  double alpha[kMaxLoads];
  bool act[kMaxLoads];
#pragma unroll
  for (int l = 0; l < kMaxLoads; ++l) {
    acc[l] = 0.;
    act[l] = l < g.L && !st[l].done;
    alpha[l] = act[l] ? st[l].alpha : 0.;
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
#pragma unroll
    for (int l = 0; l < kMaxLoads; ++l) {
      if (l >= g.L) break;
      if (!act[l]) continue;
      // updates in the field precision; <R,R> summed over the comps of a voxel
      // in the field precision, across voxels in FP64
      const R a = (R)alpha[l];
      R sq = R(0);
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const long long i = (long long)(l * g.dv + c) * g.M + v;
        x[i] = x[i] + a * p[i];
        const R rn = r[i] - a * ap[i];
        r[i] = rn;
        sq += rn * rn;
      }
      acc[l] += (double)sq;
    }
  }
  block_sum_n(acc, g.L, red, partials + (long long)blockIdx.x * g.L);
}

// The same update with the grid split by component (blockIdx.y = load * dv +
// c): each CTA streams one component's four input and two output arrays
// (instead of all components of a voxel at once) with four voxels in flight
// per thread.  Partial <R,R> go to partials[(y * gridDim.x + x) * L + l] with
// zeros for the other loads, so the finalisation over gridDim.x * gridDim.y
// parts is unchanged.
template <typename R>
__global__ void __launch_bounds__(256) k_cg_update_comp(R* __restrict__ x, R* __restrict__ r,
                                                        const R* __restrict__ p,
                                                        const R* __restrict__ ap,
                                                        double* __restrict__ partials, GridDims g,
                                                        const LoadState* __restrict__ st,
                                                        const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8];
  {  // the cell of a batched plan (grid z); partial sums [cell][y][x][load]
    const long long k = blockIdx.z;
    x += k * g.sf;
    r += k * g.sf;
    p += k * g.sf;
    ap += k * g.sf;
    st += k * g.L;
    partials += k * gridDim.x * gridDim.y * g.L;
  }
  const int comp = blockIdx.y;
  const int l = comp / g.dv;
  const bool act = !st[l].done;
  double acc = 0.;
  if (act) {
    const R a = (R)st[l].alpha;
    const long long off = (long long)comp * g.M;
    R* xc = x + off;
    R* rc = r + off;
    const R* pc = p + off;
    const R* apc = ap + off;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    R sq = R(0);
    for (; v + 3 * stride < g.M; v += 4 * stride) {
      R pv[4], av[4], xv[4], rv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        pv[u] = pc[v + u * stride];
        av[u] = apc[v + u * stride];
        xv[u] = xc[v + u * stride];
        rv[u] = rc[v + u * stride];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        xc[v + u * stride] = xv[u] + a * pv[u];
        const R rn = rv[u] - a * av[u];
        rc[v + u * stride] = rn;
        sq += rn * rn;
      }
    }
    for (; v < g.M; v += stride) {
      xc[v] = xc[v] + a * pc[v];
      const R rn = rc[v] - a * apc[v];
      rc[v] = rn;
      sq += rn * rn;
    }
    acc = (double)sq;
  }
  double t = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    double* out = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L;
    for (int k = 0; k < g.L; ++k) out[k] = k == l ? tot : 0.;
  }
}

// Finalise <P,AP>: alpha = rr / pap  (solver.py:126)
static __global__ void k_fin_pap(const double* __restrict__ partials, int nparts, LoadState* st, int L,
                          double invM, const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8];
  partials += (long long)blockIdx.y * nparts * L;   // the cell of a batched plan (grid y)
  st += (long long)blockIdx.y * L;
  const int l = blockIdx.x;
  if (st[l].done) return;
  double s = 0.;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(long long)i * L + l];
  double t = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    const double pap = tot * invM;
    st[l].pap = pap;
    if (!(pap > 0.) || !isfinite(pap)) {
      st[l].status = isfinite(pap) ? 2 : 3;
      st[l].alpha = 0.;
      st[l].done = 1;
    } else {
      st[l].alpha = st[l].rr / pap;
    }
  }
}

// Finalise <R,R>: beta, norm, kit, stopping test (solver.py:129-134,123).
// Also (first block) refreshes the all-done flag.
static __global__ void k_fin_rr(const double* __restrict__ partials, int nparts, LoadState* st, int L,
                         double invM, double* __restrict__ res_log, int log_cap, int* all_done) {
  __shared__ double red[8];
  const int l = blockIdx.x;
  if (*all_done) return;
  // the cell of a batched plan (grid y); residual log rows of gridDim.y * L
  const int cell = blockIdx.y;
  partials += (long long)cell * nparts * L;
  st += (long long)cell * L;
  const bool was_done = st[l].done;
  if (!was_done) {
    double s = 0.;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(long long)i * L + l];
    double t = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      const double rrn = tot * invM;
      LoadState& S = st[l];
      S.kit += 1;
      S.beta = rrn / S.rr;
      S.rr = rrn;
      S.norm_res = sqrt(rrn);
      if (res_log && S.kit < log_cap)
        res_log[(long long)S.kit * L * gridDim.y + (long long)cell * L + l] = S.norm_res;
      if (!isfinite(rrn)) { S.status = 3; S.done = 1; }
      if (!(S.norm_res > S.tol && S.kit < S.maxiter)) S.done = 1;
      if (S.norm_res < S.min_norm) S.min_norm = S.norm_res;
      // FP32 fields: past the precision floor the recursion can diverge; stop
      // while the iterate is still at the floor's accuracy
      if (S.guard > 0. && S.kit >= 10 && S.norm_res > S.guard * S.min_norm) {
        S.status = 1;
        S.done = 1;
      }
    }
  }
}

// all_done = AND over loads (run after k_fin_rr, one thread)
static __global__ void k_update_all_done(const LoadState* st, int L, int* all_done) {
  int d = 1;
  for (int l = 0; l < L; ++l) d &= st[l].done;
  *all_done = d;
}

// initial residual norms: rr = sum/M, norm = sqrt(rr), done = !(norm > tol && 0 < maxiter)
static __global__ void k_fin_init(const double* __restrict__ partials, int nparts, LoadState* st, int L,
                           double invM, double* __restrict__ res_log, int log_cap) {
  const int l = threadIdx.x;
  if (l >= L) return;
  // the cell of a batched plan (grid x); residual log rows of gridDim.x * L
  const int cell = blockIdx.x;
  partials += (long long)cell * nparts * L;
  st += (long long)cell * L;
  if (res_log) res_log += (long long)cell * L;
  double s = 0.;
  for (int i = 0; i < nparts; ++i) s += partials[(long long)i * L + l];
  LoadState& S = st[l];
  S.rr = s * invM;
  S.norm_res = sqrt(S.rr);
  S.min_norm = S.norm_res;
  S.kit = 0;
  S.beta = 0.;
  S.alpha = 0.;
  S.status = isfinite(S.rr) ? 0 : 3;
  S.done = !(S.norm_res > S.tol && 0 < S.maxiter) || S.status != 0;
  if (res_log && log_cap > 0) res_log[l] = S.norm_res;
}

// y = a*x + b*y elementwise over n values, in the field precision (FP64
// arithmetic is the slow pipe on this GPU)
template <typename R>
__global__ void k_axpby(long long n, double a, const R* __restrict__ x, double b, R* __restrict__ y) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const R ar = (R)a, br = (R)b;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = ar * x[i] + br * y[i];
}

// x[l*dv + c] = val * delta(c, l)  (the constant macroscopic field E_N of load l,
// ffthompy/applications.py:60-65, with val = -1 for the right-hand side)
template <typename R>
__global__ void k_fill_macro(R* __restrict__ x, GridDims g, double val) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tot = (long long)g.K * g.L * g.dv * g.M;   // every cell of a batched plan
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    const long long comp = i / g.M;
    const long long j = comp / g.dv;
    const int c = (int)(comp - j * g.dv), l = (int)(j % g.L);
    x[i] = (c == l) ? (R)val : R(0);
  }
}

// A_H partials: sum_v <A(v) u_i(v), u_j(v)>, u_i = X_i + e_i (postprocess.py:53-70,
// add_macro2minimizer 73-86).  L <= 6 loads -> 36 accumulators.
template <typename R, int COEF>
__global__ void __launch_bounds__(128) k_energy(const R* __restrict__ X, const R* __restrict__ A,
                                                double* __restrict__ partials, GridDims g,
                                                int add_macro) {
  {  // the cell of a batched plan (grid y); partial sums [cell][CTA][L * L]
    const long long k = blockIdx.y;
    X += k * g.sf;
    A += k * g.sa;
    partials += k * gridDim.x * g.L * g.L;
  }
  __shared__ double red[4 * kMaxLoads * kMaxLoads];
  const int L = g.L, dv = g.dv;
  double acc[kMaxLoads * kMaxLoads];
  for (int i = 0; i < kMaxLoads * kMaxLoads; ++i) acc[i] = 0.;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
    R u[kMaxLoads][kMaxDv];
    for (int l = 0; l < L; ++l)
      for (int c = 0; c < dv; ++c)
        u[l][c] = X[(long long)(l * dv + c) * g.M + v] + ((add_macro && c == l) ? R(1) : R(0));
    for (int i = 0; i < L; ++i) {
      R q[kMaxDv];
      coef_apply<R, COEF>(A, g.M, v, dv, u[i], q);
      for (int j = 0; j < L; ++j) {
        double s = 0.;
        for (int c = 0; c < dv; ++c) s += (double)q[c] * (double)u[j][c];
        acc[i * L + j] += s;
      }
    }
  }
  block_sum_n(acc, L * L, red, partials + (long long)blockIdx.x * L * L);
}

// Load-pair weights of a scalar function of A_H (the adjoint seed dF/dA_H).
struct LoadMat {
  double w[kMaxLoads * kMaxLoads];
};

// Coefficient gradient of sum_ij W[i][j] A_H[i][j], A_H[i][j] = <A u_i, u_j> =
// (1/M) sum_v u_j(v) . A(v) u_i(v), u_i = X_i (+ E_i).  At the solution of
// G A u_i = 0 the fields are stationary (Galerkin orthogonality), so the
// derivative is the explicit one and needs no adjoint solve:
//   S_ab(v) = sum_ij W_ij u_j[a] u_i[b] / M
//   ISO: sum_a S_aa;  SYM (packed a <= b): S_aa, S_ab + S_ba;  FULL: S_ab.
// FP64 throughout (a one-off per gradient).
template <typename R, int COEF>
__global__ void __launch_bounds__(128) k_energy_grad(const R* __restrict__ X,
                                                     double* __restrict__ grad,
                                                     const __grid_constant__ GridDims g,
                                                     int add_macro,
                                                     const __grid_constant__ LoadMat W,
                                                     double invM) {
  const int L = g.L, dv = g.dv;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
    double u[kMaxLoads][kMaxDv], T[kMaxLoads][kMaxDv];
#pragma unroll
    for (int l = 0; l < kMaxLoads; ++l)
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        u[l][c] = (l < L && c < dv) ? (double)X[(long long)(l * dv + c) * g.M + v] +
                                          ((add_macro && c == l) ? 1. : 0.)
                                    : 0.;
      }
    // T[j][b] = sum_i W_ij u_i[b]
#pragma unroll
    for (int j = 0; j < kMaxLoads; ++j)
#pragma unroll
      for (int b = 0; b < kMaxDv; ++b) {
        double t = 0.;
#pragma unroll
        for (int i = 0; i < kMaxLoads; ++i)
          if (i < L && j < L) t += W.w[i * L + j] * u[i][b];
        T[j][b] = t;
      }
    auto S = [&](int a, int b) {
      double s = 0.;
#pragma unroll
      for (int j = 0; j < kMaxLoads; ++j) s += u[j][a] * T[j][b];
      return s * invM;
    };
    if constexpr (COEF == COEF_ISO) {
      double s = 0.;
#pragma unroll
      for (int a = 0; a < kMaxDv; ++a)
        if (a < dv) s += S(a, a);
      grad[v] = s;
    } else if constexpr (COEF == COEF_SYM) {
#pragma unroll
      for (int a = 0; a < kMaxDv; ++a)
#pragma unroll
        for (int b = 0; b < kMaxDv; ++b) {
          if (a < dv && b < dv && a <= b) {
            const int t = a * dv - a * (a - 1) / 2 + (b - a);
            grad[(long long)t * g.M + v] = a == b ? S(a, a) : S(a, b) + S(b, a);
          }
        }
    } else {
#pragma unroll
      for (int a = 0; a < kMaxDv; ++a)
#pragma unroll
        for (int b = 0; b < kMaxDv; ++b)
          if (a < dv && b < dv) grad[(long long)(a * dv + b) * g.M + v] = S(a, b);
    }
  }
}

// sum partials[nparts][n] -> out[n] (one block)
static __global__ void k_sum_partials(const double* __restrict__ partials, int nparts, int n,
                               double scale, double* __restrict__ out) {
  partials += (long long)blockIdx.x * nparts * n;   // the cell of a batched plan (grid x)
  out += (long long)blockIdx.x * n;
  for (int j = 0; j < n; ++j) {
    double s = 0.;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(long long)i * n + j];
    __shared__ double red[32];
    double t = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      out[j] = tot * scale;
    }
    __syncthreads();
  }
}

// Trigonometric interpolation N -> M on half spectra (Tensor.enlarge,
// ffthompy/tensors/objects.py:428-467): target coefficient at signed
// frequency q takes the source coefficient at q (weight 1) when |q| < N/2,
// half of the Nyquist coefficient when N is even and |q| = N/2, else 0.
template <typename R>
__global__ void k_spectrum_pad(const cplx<R>* __restrict__ Sn, cplx<R>* __restrict__ Sm,
                               int C, int dim, int N0, int N1, int N2, int M0, int M1, int M2) {
  const int N2h = N2 / 2 + 1, M2h = M2 / 2 + 1;
  const long long tot = (long long)C * M0 * M1 * M2h;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    long long r = i;
    const int k2 = (int)(r % M2h); r /= M2h;
    const int k1 = (int)(r % M1); r /= M1;
    const int k0 = (int)(r % M0); r /= M0;
    const int c = (int)r;
    double w = 1.;
    int src[3];
    const int Ms[2] = {M0, M1}, Ns[2] = {N0, N1}, ks[2] = {k0, k1};
    bool ok = true;
    for (int a = 0; a < 2; ++a) {
      const int q = signed_freq(ks[a], Ms[a]);
      const int Na = Ns[a];
      const int aq = q < 0 ? -q : q;
      if (2 * aq < Na) src[a] = q < 0 ? q + Na : q;
      else if (2 * aq == Na) { src[a] = Na / 2; w *= 0.5; }
      else { ok = false; break; }
    }
    if (ok) {
      if (2 * k2 < N2) src[2] = k2;
      else if (2 * k2 == N2) { src[2] = N2 / 2; w *= 0.5; }
      else ok = false;
    }
    cplx<R> v = mkc<R>(R(0), R(0));
    if (ok) {
      const cplx<R> s = Sn[(((long long)c * N0 + src[0]) * N1 + src[1]) * N2h + src[2]];
      v = mkc<R>((R)(w * (double)s.x), (R)(w * (double)s.y));
    }
    Sm[i] = v;
  }
}

// Ga grid-based coefficient spectrum (ffthompy/materials.py:77-110): target
// half-spectrum entry (t0,t1,t2) of the 2N-1 grid takes the source DFT
// coefficient at (src0[t0], src1[t1], src2[t2]) of the P-grid image (the
// reference's periodic tiling + central crop, as per-axis index tables) times
// the separable cell-shape weights w0[t0] w1[t1] w2[t2].  Sources outside the
// stored half spectrum are read through Hermitian symmetry.
template <typename R>
__global__ void k_ga_gather(const cplx<R>* __restrict__ Sp, cplx<R>* __restrict__ St, int C,
                            int P0, int P1, int P2, int T0, int T1, int T2,
                            const int* __restrict__ src, const double* __restrict__ w) {
  const int P2h = P2 / 2 + 1, T2h = T2 / 2 + 1;
  const int* s0 = src;
  const int* s1 = src + T0;
  const int* s2 = src + T0 + T1;
  const double* w0 = w;
  const double* w1 = w + T0;
  const double* w2 = w + T0 + T1;
  const long long tot = (long long)C * T0 * T1 * T2h;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    long long r = i;
    const int t2 = (int)(r % T2h); r /= T2h;
    const int t1 = (int)(r % T1); r /= T1;
    const int t0 = (int)(r % T0); r /= T0;
    const int c = (int)r;
    int a0 = s0[t0], a1 = s1[t1], a2 = s2[t2];
    bool conj = false;
    if (a2 >= P2h) {  // X[a] = conj(X[-a])
      a2 = P2 - a2;
      a0 = a0 ? P0 - a0 : 0;
      a1 = a1 ? P1 - a1 : 0;
      conj = true;
    }
    cplx<R> v = Sp[(((long long)c * P0 + a0) * P1 + a1) * P2h + a2];
    if (conj) v.y = -v.y;
    const double ww = w0[t0] * w1[t1] * w2[t2];
    St[i] = mkc<R>((R)(ww * (double)v.x), (R)(ww * (double)v.y));
  }
}

// ---------------------------------------------------------------------------
// Band representation of the Ga operator (CG fields on the solve grid N, the
// coefficient applied on an integration grid B >= 2N-1).  Along one axis:
//   BAND_UP        : space N  -> DFT_N -> band |k| <= h -> iDFT_B -> space B
//   BAND_DOWN      : space B  -> DFT_B -> band -> frequency (N layout)
//   BAND_DOWN_PROJ : space B  -> DFT_B -> band -> G(xi) over the dv comps ->
//                    iDFT_N -> space N
// Arrays are [comp][mid][axis][inner]; CTA = T inner columns of one (comp, mid)
// (of one (load, mid) with all dv comps for BAND_DOWN_PROJ).
// ---------------------------------------------------------------------------
//   BAND_UP_PROJ   : space N  -> DFT_N -> G(xi) -> iDFT_B (band pad) -> space B
//   BAND_PAD       : frequency (N layout) -> band pad -> iDFT_B -> space B
//   BAND_PAD_PUPD  : as BAND_PAD, the input being the CG direction of the
//                    spectral iterates, updated first (p = r + beta p)
//   BAND_DOWN_F    : space B -> DFT_B -> band -> times the operator scale ->
//                    frequency (N layout) of the spectral iterates, with the
//                    partial <p, Ap>; the spectral CG applies G in its update
enum BandMode { BAND_UP = 0, BAND_DOWN = 1, BAND_DOWN_PROJ = 2, BAND_UP_PROJ = 3, BAND_PAD = 4,
                BAND_PAD_PUPD = 5, BAND_DOWN_F = 7 };

struct BandAxis {
  int n_in, n_out;     // line lengths in / out
  int nN, nB;          // solve / integration length of this axis
  int h;               // band half width
  long long inner;     // contiguous elements after the axis
  int mid;             // extent of the axis before this one (1 if none)
  int mid_n;           // N extent of the mid axis (its frequency layout), PROJ only
  int pmode;           // frequency decoding for G: 0 2D (line, inner); 1 3D (mid, line,
                       // inner); 2 3D (line, inner = k1 * inner2 + k2)
  int inner2;          // pmode 2: extent of the last axis (half spectrum)
  int n1f;             // pmode 2: N extent of axis 1 (frequency layout)
  FastDiv dn_in, dn_out, dinner2;  // division by n_in, n_out, inner2
};

inline void set_band_divs(BandAxis& ax) {
  ax.dn_in = make_fastdiv((unsigned)ax.n_in);
  ax.dn_out = make_fastdiv((unsigned)ax.n_out);
  ax.dinner2 = make_fastdiv((unsigned)(ax.inner2 > 0 ? ax.inner2 : 1));
}

__device__ __forceinline__ void band_freqs(const BandAxis& ax, int dim, int q, int m,
                                           long long col, int* kv) {
  if (dim == 2) { kv[0] = q; kv[1] = (int)col; return; }
  if (ax.pmode == 1) { kv[0] = signed_freq(m, ax.mid_n); kv[1] = q; kv[2] = (int)col; return; }
  const int k1 = fdiv((int)col, ax.dinner2);
  kv[0] = q;
  kv[1] = signed_freq(k1, ax.n1f);
  kv[2] = (int)col - k1 * ax.inner2;
}

// N-layout coefficient k (grid n) from the forward B-line (length nb)
template <typename R>
__device__ __forceinline__ cplx<R> band_down_value(const cplx<R>* line, const LineDev<R>& L, int k,
                                                   int n, int nb) {
  const int q = signed_freq(k, n);
  if (2 * q == n) {  // Nyquist of an even N grid
    const cplx<R> a = get_fwd<R>(line, L, q);
    const cplx<R> b = get_fwd<R>(line, L, nb - q);
    return mkc<R>(R(0.5) * (a.x + b.x), R(0.5) * (a.y + b.y));
  }
  return get_fwd<R>(line, L, q < 0 ? q + nb : q);
}

// Spectral CG iterates are half spectra scaled to z = sqrt(w) V / prod(N), w
// the weight of the half-spectrum inner product (1 on the k2 = 0 plane and on
// the Nyquist plane of an even n2, 2 elsewhere), so that the grid-mean inner
// product of the fields is the Euclidean one of z.  Column col of a band pass
// holds last-axis frequency k2 = col mod inner2 (inner2 = n2h; 0: k2 = col).
template <typename R>
__device__ __forceinline__ R half_weight_root(const BandAxis& ax, const GridDims& g, long long col,
                                              bool inverse) {
  int k2 = (int)col;
  if (ax.inner2 > 0) k2 = (int)col - fdiv((int)col, ax.dinner2) * ax.inner2;
  if (k2 == 0 || 2 * k2 == g.n2) return R(1);
  return inverse ? R(0.70710678118654752440084436210485) : R(1.4142135623730950488016887242097);
}

// forward output slot of frequency k written so that get_fwd returns v
template <typename R>
__device__ __forceinline__ void set_fwd(cplx<R>* line, const LineDev<R>& L, int k, cplx<R> v) {
  if (L.blue) line[sp(k)] = cmulc<R>(v, L.chirp[k]);
  else line[sp(line_pos<R>(L, k))] = v;
}

// Visits every (tile line c < nlc, line index k < n, column t < T) of a
// column tile once.  When T divides the block, a thread keeps one column t and
// walks k with a fixed stride, so no index is divided per element and the
// per-line bases are loop invariants; body(c, k, t).
template <typename F>
__device__ __forceinline__ void tile_loop(int nlc, int n, int T, int lgT, F&& body) {
  if (T <= (int)blockDim.x) {
    const int t = threadIdx.x & (T - 1);
    const int kst = (int)blockDim.x >> lgT;
    const int k0 = (int)threadIdx.x >> lgT;
    for (int c = 0; c < nlc; ++c)
      for (int k = k0; k < n; k += kst) body(c, k, t);
  } else {
    for (int e = threadIdx.x; e < nlc * n * T; e += blockDim.x) {
      const int t = e & (T - 1), rest = e >> lgT;
      const int c = rest / n, k = rest - c * n;
      body(c, k, t);
    }
  }
}

// aux: BAND_PAD_PUPD the CG direction p (read and updated in place, Sin = r);
// BAND_DOWN_F the direction p read for the partial <p, Ap>, written to
// partials[(blockIdx.y * gridDim.x + blockIdx.x) * L + l] (zero for l other
// than the CTA's load) when partials is not null.
// The FP32 pad and down passes of the spectral CG hold one line buffer per
// column and no per-frequency projection: three CTAs per SM fit their
// registers (80) and shared memory, which hides more of their global-memory
// latency (measured at the 509^3 workload: pad 1.13 -> 1.06 ms and 0.99 ->
// 0.85 ms; with table-free line slots, down 0.98 -> 0.92 ms and 0.63 -> 0.56).
template <typename R, int MODE>
constexpr int band_axis_min_blocks() {
  return (sizeof(R) == 4 && (MODE == BAND_PAD || MODE == BAND_PAD_PUPD || MODE == BAND_DOWN ||
                             MODE == BAND_DOWN_F))
             ? 3
             : kFftMinBlocks<R>;
}

template <typename R, int MODE, int PHYS>
__global__ void __launch_bounds__(256, band_axis_min_blocks<R, MODE>()) k_band_axis(const cplx<R>* __restrict__ Sin,
                                                   cplx<R>* __restrict__ Sout, const __grid_constant__ GridDims g,
                                                   const __grid_constant__ BandAxis ax, const __grid_constant__ LineDev<R> L1, const __grid_constant__ LineDev<R> L2,
                                                   int T, const __grid_constant__ GreenParams gp,
                                                   const int* __restrict__ all_done,
                                                   const LoadState* __restrict__ st,
                                                   cplx<R>* __restrict__ aux,
                                                   double* __restrict__ partials) {
  if (all_done && *all_done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool PROJ = (MODE == BAND_DOWN_PROJ || MODE == BAND_UP_PROJ);
  constexpr bool PADIN = (MODE == BAND_PAD || MODE == BAND_PAD_PUPD);
  const int nlc = PROJ ? g.dv : 1;   // comps per CTA
  // blockIdx.y: (comp or load) * mid + m
  const int m = blockIdx.y % ax.mid;
  const int cl = blockIdx.y / ax.mid;
  const int c0 = PROJ ? cl * g.dv : cl;
  const int load = c0 / g.dv;
  if (st && st[load].done) {
    if (MODE == BAND_DOWN_F && partials && threadIdx.x < g.L)
      partials[((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L + threadIdx.x] = 0.;
    return;
  }
  const int ld1 = PADIN ? 0 : L1.ld;
  const int ld2 = (MODE == BAND_DOWN || MODE == BAND_DOWN_F) ? 0 : L2.ld;
  cplx<R>* buf1 = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* buf2 = buf1 + (size_t)nlc * T * ld1;
  const long long t0 = (long long)blockIdx.x * T;
  const int nl = nlc * T;
  const int lgT = __ffs(T) - 1;  // T is a power of two
  // band-pruned power-of-two B lines (line_prunable): the up / pad inverse
  // transforms see at most |q| <= n_in/2 nonzero, the down forward transforms
  // are read at |q| <= n_out/2 only; zeros on the pruned digits are not written
  const bool pr2 = (MODE == BAND_UP || MODE == BAND_UP_PROJ || PADIN) &&
                   line_prunable<R>(L2, ax.n_in / 2);
  const bool pr1 = (MODE == BAND_DOWN || MODE == BAND_DOWN_PROJ || MODE == BAND_DOWN_F) &&
                   line_prunable<R>(L1, ax.n_out / 2);
  const int pq0 = L2.nf / 4, pq1 = 3 * (L2.nf / 4);  // pruned range of the B line (pr2)
  if constexpr (MODE == BAND_PAD) {
    // input already in frequency (N layout): pad straight into the B line
    // raw values go straight to the inverse-input slots (plain async copies
    // inside the band; the halved Nyquist entry and zeros by ordinary stores)
    tile_loop(1, ax.n_out, T, lgT, [&](int, int k, int t) {
      if (pr2 && k >= pq0 && k < pq1) return;
      const long long col = t0 + t;
      const int q = signed_freq(k, ax.n_out);
      const int aq = q < 0 ? -q : q;
      cplx<R>* slot = buf2 + t * ld2 + slot_inv<R>(L2, k);
      const cplx<R>* src = Sin + (((long long)c0 * ax.mid + m) * ax.n_in) * ax.inner + col;
      if (col < ax.inner && 2 * aq < ax.n_in) {
        cp_async_cplx<R>(slot, src + (long long)(q < 0 ? q + ax.n_in : q) * ax.inner);
      } else if (col < ax.inner && 2 * aq == ax.n_in) {
        *slot = cscale<R>(src[(long long)aq * ax.inner], R(0.5));
      } else {
        *slot = mkc<R>(R(0), R(0));
      }
    });
    cp_async_commit();
    cp_async_wait<0>();
  } else if constexpr (MODE == BAND_PAD_PUPD) {
    // p = r + beta p on the spectral iterates (Sin = r, aux = p, N layout,
    // updated in place), then p / sqrt(w) padded into the B line.  Entries
    // with 2|q| = n_in (the Nyquist index of an even n_in) are zero on
    // range(G), where the iterates live, and stay untouched.
    const R bet = R(st[load].beta);
    const cplx<R>* rbase = Sin + (((long long)c0 * ax.mid + m) * ax.n_in) * ax.inner + t0;
    cplx<R>* pbase = aux + (((long long)c0 * ax.mid + m) * ax.n_in) * ax.inner + t0;
    if (pr2 && !L2.blue) {
      // pruned direct B lines: the slots of the pruned frequencies
      // [nf/4, 3nf/4) are never read by the inverse core, so they hold r
      // while p sits in its own slot; both arrive by cp.async (all loads in
      // flight at once), then p is updated, written back and scaled in place
      const int sh = L2.nf / 4;
      tile_loop(1, ax.n_out, T, lgT, [&](int, int k, int t) {
        if (k >= pq0 && k < pq1) return;
        const int q = signed_freq(k, ax.n_out);
        const int aq = q < 0 ? -q : q;
        cplx<R>* slot = buf2 + t * ld2 + slot_inv<R>(L2, k);
        if (t0 + t < ax.inner && 2 * aq < ax.n_in) {
          const long long off = (long long)(q < 0 ? q + ax.n_in : q) * ax.inner + t;
          cp_async_cplx<R>(slot, pbase + off);
          cp_async_cplx<R>(buf2 + t * ld2 + slot_inv<R>(L2, q < 0 ? k - sh : k + sh), rbase + off);
        } else {
          *slot = mkc<R>(R(0), R(0));
        }
      });
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      tile_loop(1, ax.n_out, T, lgT, [&](int, int k, int t) {
        if (k >= pq0 && k < pq1) return;
        const int q = signed_freq(k, ax.n_out);
        const int aq = q < 0 ? -q : q;
        const long long col = t0 + t;
        if (col < ax.inner && 2 * aq < ax.n_in) {
          cplx<R>* slot = buf2 + t * ld2 + slot_inv<R>(L2, k);
          const cplx<R> r = buf2[t * ld2 + slot_inv<R>(L2, q < 0 ? k - sh : k + sh)];
          cplx<R> p = *slot;
          p = mkc<R>(r.x + bet * p.x, r.y + bet * p.y);
          pbase[(long long)(q < 0 ? q + ax.n_in : q) * ax.inner + t] = p;
          *slot = cscale<R>(p, half_weight_root<R>(ax, g, col, true));
        }
      });
    } else {
      tile_loop(1, ax.n_out, T, lgT, [&](int, int k, int t) {
        if (pr2 && k >= pq0 && k < pq1) return;
        const long long col = t0 + t;
        const int q = signed_freq(k, ax.n_out);
        const int aq = q < 0 ? -q : q;
        cplx<R> v = mkc<R>(R(0), R(0));
        if (col < ax.inner && 2 * aq < ax.n_in) {
          const long long off = (long long)(q < 0 ? q + ax.n_in : q) * ax.inner + t;
          const cplx<R> r = rbase[off];
          cplx<R> p = pbase[off];
          p = mkc<R>(r.x + bet * p.x, r.y + bet * p.y);
          pbase[off] = p;
          v = cscale<R>(p, half_weight_root<R>(ax, g, col, true));
        }
        buf2[t * ld2 + slot_inv<R>(L2, k)] = v;
      });
    }
  } else {
    // load: [comp][mid][n_in][inner]
    tile_loop(nlc, ax.n_in, T, lgT, [&](int c, int i, int t) {
      const long long col = t0 + t;
      const cplx<R>* src = Sin + (((long long)(c0 + c) * ax.mid + m) * ax.n_in) * ax.inner + col;
      cplx<R>* slot = buf1 + (c * T + t) * ld1 + slot_fwd<R>(L1, i);
      if (col < ax.inner) cp_async_cplx<R>(slot, src + (long long)i * ax.inner);
      else *slot = mkc<R>(R(0), R(0));
    });
    cp_async_commit();
    zero_tail<R>(buf1, ld1, nl, L1);
    cp_async_wait<0>();
    __syncthreads();
    if (L1.blue) {
      blue_fixup<R, false>(buf1, ld1, nl, L1);
      __syncthreads();
    }
    line_core<R>(buf1, ld1, nl, L1, false, pr1);
  }
  // Up: the B-grid coefficient at q is the N-grid one for 2|q| < N, half of the
  // Nyquist one for 2|q| = N (the symmetric split of Tensor.enlarge,
  // ffthompy/tensors/objects.py:441-453), else 0.  Down (the adjoint): the
  // N-grid coefficient at k is the B-grid one for 2|k| < N and the mean of the
  // B-grid coefficients at +-N/2 for the Nyquist index.
  if constexpr (MODE == BAND_UP_PROJ) {
    // G over the dv comps of each N frequency, then the padded B line.  Lanes
    // take consecutive frequencies of one column: the digit-reversed slots of
    // consecutive k fall in distinct banks, those of one k in the T lines of a
    // column tile do not.
    for (int t = 0; t < T; ++t)
    for (int k = threadIdx.x; k < ax.n_in; k += blockDim.x) {
      const long long col = t0 + t;
      const int q = signed_freq(k, ax.n_in);
      cplx<R> x[kMaxDv];
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c)
        if (c < g.dv) x[c] = get_fwd<R>(buf1 + (c * T + t) * ld1, L1, k);
      if (col < ax.inner) {
        int kv[3];
        band_freqs(ax, g.dim, q, m, col, kv);
        green_apply<R, PHYS>(gp, g.dim, kv, x);
      }
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        // the projected spectrum is band limited (Nyquist zeroed): place it
        cplx<R>* l2 = buf2 + (c * T + t) * ld2;
        if (2 * (q < 0 ? -q : q) < ax.n_in) put_inv<R>(l2, L2, q < 0 ? q + ax.n_out : q, x[c]);
      }
    }
    // the remaining B frequencies are zero
    {
      // out-of-band frequencies only (2|q| >= n_in): k in [kb, n_out - kb]
      const int kb = (ax.n_in + 1) / 2, ke = ax.n_out - kb + 1;
      tile_loop(nlc, ke - kb, T, lgT, [&](int c, int kk, int t) {
        if (pr2 && kb + kk >= pq0 && kb + kk < pq1) return;
        put_inv<R>(buf2 + (c * T + t) * ld2, L2, kb + kk, mkc<R>(R(0), R(0)));
      });
    }
  }
  if constexpr (MODE == BAND_UP || MODE == BAND_UP_PROJ || PADIN) {
    if constexpr (MODE == BAND_UP) {
    tile_loop(nlc, ax.n_out, T, lgT, [&](int c, int k, int t) {
      if (pr2 && k >= pq0 && k < pq1) return;
      const int line = c * T + t;
      const int q = signed_freq(k, ax.n_out);
      const int aq = q < 0 ? -q : q;
      cplx<R> v = mkc<R>(R(0), R(0));
      if (2 * aq < ax.n_in) {
        v = get_fwd<R>(buf1 + line * ld1, L1, q < 0 ? q + ax.n_in : q);
      } else if (2 * aq == ax.n_in) {
        v = cscale<R>(get_fwd<R>(buf1 + line * ld1, L1, aq), R(0.5));
      }
      put_inv<R>(buf2 + line * ld2, L2, k, v);
    });
    }
    __syncthreads();
    if constexpr (PADIN) blue_fixup<R, true>(buf2, ld2, nl, L2);
    zero_tail<R>(buf2, ld2, nl, L2);
    __syncthreads();
    line_core<R>(buf2, ld2, nl, L2, true, pr2);
    tile_loop(nlc, ax.n_out, T, lgT, [&](int c, int i, int t) {
      const long long col = t0 + t;
      if (col >= ax.inner) return;
      cplx<R>* dst = Sout + (((long long)(c0 + c) * ax.mid + m) * ax.n_out) * ax.inner + col;
      dst[(long long)i * ax.inner] = get_inv<R>(buf2 + (c * T + t) * ld2, L2, i);
    });
  } else if constexpr (MODE == BAND_DOWN) {
    tile_loop(nlc, ax.n_out, T, lgT, [&](int c, int k, int t) {
      const long long col = t0 + t;
      if (col >= ax.inner) return;
      const cplx<R> v = band_down_value<R>(buf1 + (c * T + t) * ld1, L1, k, ax.n_out, ax.n_in);
      cplx<R>* dst = Sout + (((long long)(c0 + c) * ax.mid + m) * ax.n_out) * ax.inner + col;
      dst[(long long)k * ax.inner] = v;
    });
  } else if constexpr (MODE == BAND_DOWN_F) {
    // rows of T columns to global (z form: times sqrt(w) and the operator's
    // scale s / prod(B)), with <p, Ap>: a thread keeps one column and takes
    // its frequencies four at a time, the four loads of p issued before their
    // products.  The Nyquist index of an even N takes the mean of the B-line
    // coefficients at +-N/2 (band_down_value): CG iterates have none there,
    // the energies of arbitrary fields do.
    const R osc = R(gp.scale);
    R dot = R(0);
    if (T <= (int)blockDim.x) {
      const int t = threadIdx.x & (T - 1);
      const int kst = (int)blockDim.x >> lgT;
      const long long col = t0 + t;
      if (col < ax.inner) {
        const R fo = half_weight_root<R>(ax, g, col, false) * osc;
        for (int c = 0; c < nlc; ++c) {
          const long long base = (((long long)(c0 + c) * ax.mid + m) * ax.n_out) * ax.inner + col;
          const cplx<R>* line = buf1 + (c * T + t) * ld1;
          for (int k = (int)threadIdx.x >> lgT; k < ax.n_out; k += 4 * kst) {
            cplx<R> pv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int ku = k + u * kst;
              pv[u] = (partials && ku < ax.n_out) ? aux[base + (long long)ku * ax.inner]
                                                  : mkc<R>(R(0), R(0));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int ku = k + u * kst;
              if (ku >= ax.n_out) break;
              const cplx<R> v = cscale<R>(band_down_value<R>(line, L1, ku, ax.n_out, ax.n_in), fo);
              Sout[base + (long long)ku * ax.inner] = v;
              dot += pv[u].x * v.x + pv[u].y * v.y;
            }
          }
        }
      }
    } else {
      tile_loop(nlc, ax.n_out, T, lgT, [&](int c, int k, int t) {
        const long long col = t0 + t;
        if (col >= ax.inner) return;
        cplx<R> v = band_down_value<R>(buf1 + (c * T + t) * ld1, L1, k, ax.n_out, ax.n_in);
        v = cscale<R>(v, half_weight_root<R>(ax, g, col, false) * osc);
        const long long idx = (((long long)(c0 + c) * ax.mid + m) * ax.n_out + k) * ax.inner + col;
        Sout[idx] = v;
        if (partials) {
          const cplx<R> p = aux[idx];
          dot += p.x * v.x + p.y * v.y;
        }
      });
    }
    if (partials) {
      // the line buffers are read: their first bytes take the warp sums (no
      // static shared memory, so the whole dynamic allowance stays usable)
      __syncthreads();
      double* red = reinterpret_cast<double*>(smem_raw);
      const double tsum = warp_sum((double)dot);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = tsum;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
        double* out = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L;
        for (int l = 0; l < g.L; ++l) out[l] = l == load ? tot : 0.;
      }
    }
  } else {
    // G(xi) on the band, then inverse DFT_N along the line (lanes over the
    // frequencies of one column, as in the up projection)
    for (int t = 0; t < T; ++t)
    for (int k = threadIdx.x; k < ax.n_out; k += blockDim.x) {
      const long long col = t0 + t;
      const int q = signed_freq(k, ax.n_out);
      cplx<R> x[kMaxDv];
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c)
        if (c < g.dv) x[c] = band_down_value<R>(buf1 + (c * T + t) * ld1, L1, k, ax.n_out, ax.n_in);
      if (col < ax.inner) {
        int kv[3];
        band_freqs(ax, g.dim, q, m, col, kv);
        green_apply<R, PHYS>(gp, g.dim, kv, x);
      }
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c)
        if (c < g.dv) put_inv<R>(buf2 + (c * T + t) * ld2, L2, k, x[c]);
    }
    zero_tail<R>(buf2, ld2, nl, L2);
    __syncthreads();
    line_core<R>(buf2, ld2, nl, L2, true);
    tile_loop(nlc, ax.n_out, T, lgT, [&](int c, int i, int t) {
      const long long col = t0 + t;
      if (col >= ax.inner) return;
      cplx<R>* dst = Sout + (((long long)(c0 + c) * ax.mid + m) * ax.n_out) * ax.inner + col;
      dst[(long long)i * ax.inner] = get_inv<R>(buf2 + (c * T + t) * ld2, L2, i);
    });
  }
}

// Shared-memory layout of k_band_last (host and device use the same sizes):
// [pair lines rows*np*ld | staged band spectra C*rows*n2h | staged coefficient
// cA*rows*n2], each region starting on a 16-byte boundary.
// stage: bit 0 stages the band spectra, bit 1 the coefficient (each only when
// it fits next to the lines; otherwise the phase reads global memory).
template <typename R>
__host__ __device__ inline size_t band_last_smem_bytes(int rows, int np, int ld, int C, int n2h,
                                                       int cA, int n2, int stage) {
  return align16((size_t)rows * np * ld * sizeof(cplx<R>)) +
         ((stage & 1) ? align16((size_t)C * rows * n2h * sizeof(cplx<R>)) : 0) +
         ((stage & 2) ? (size_t)cA * rows * n2 * sizeof(R) : 0);
}
template <int COEF>
__host__ __device__ constexpr int coef_comps(int dv) {
  return COEF == COEF_ISO ? 1 : COEF == COEF_SYM ? dv * (dv + 1) / 2 : dv * dv;
}

// Last axis on the integration grid, in place on band half spectra
// S[comp][row][N2h] (row over the B grid's leading axes): c2r to the B2 points,
// q = A x * cscale per voxel, r2c back and keep the band k2 <= h2.
template <typename R, int COEF>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_band_last(cplx<R>* __restrict__ S,
                                                   const R* __restrict__ A, const __grid_constant__ GridDims g,
                                                   long long nrows, int n2h_band, int n2_solve,
                                                   const __grid_constant__ LineDev<R> L, int rows, R coef_scale,
                                                   const int* __restrict__ all_done, int stage) {
  if (all_done && *all_done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int C = g.L * g.dv;
  const int np = (C + 1) / 2;
  const int ld = L.ld;
  const int n = L.n;                       // B2
  const long long Mi = nrows * n;          // voxels of the integration grid
  const long long row0 = (long long)blockIdx.x * rows;
  const int cA = coef_comps<COEF>(g.dv);
  // 0) stage this CTA's band spectra (C contiguous runs of vrows*n2h) and its
  // coefficient rows into shared memory; the coefficient group completes while
  // the inverse transforms run
  const int vrows = (int)((nrows - row0) < rows ? (nrows - row0) : rows);
  cplx<R>* sraw = reinterpret_cast<cplx<R>*>(
      smem_raw + align16((size_t)rows * np * ld * sizeof(cplx<R>)));
  R* acache = reinterpret_cast<R*>(
      reinterpret_cast<unsigned char*>(sraw) +
      ((stage & 1) ? align16((size_t)C * rows * n2h_band * sizeof(cplx<R>)) : 0));
  const bool st_spec = stage & 1, st_coef = stage & 2;
  if (st_spec)
    for (int c = 0; c < C; ++c)
      stage_async(sraw + (size_t)c * rows * n2h_band,
                  S + ((long long)c * nrows + row0) * n2h_band, vrows * n2h_band);
  cp_async_commit();
  if (st_coef)
    for (int t = 0; t < cA; ++t)
      stage_async(acache + (size_t)t * rows * n, A + (long long)t * Mi + row0 * n, vrows * n);
  cp_async_commit();
  cp_async_wait<1>();
  __syncthreads();
  // band spectrum of (comp, row rl) at frequency index aq, staged or global
  auto spec_at = [&](int comp, int rl, int aq) -> cplx<R> {
    return st_spec ? sraw[((size_t)comp * rows + rl) * n2h_band + aq]
                   : S[((long long)comp * nrows + row0 + rl) * n2h_band + aq];
  };
  // 1) Hermitian pair lines Z = A + iB over all B2 frequencies.  Frequency-
  // stationary: a thread decodes frequency k (weight, slot, chirp) once and
  // fills it in its share of the lines.
  const int nlines = rows * np;
  {
    int k0 = threadIdx.x, kstep = blockDim.x, l0 = 0, lstep = 1;
    if (n < (int)blockDim.x) {
      lstep = blockDim.x / n;
      l0 = threadIdx.x / n;
      k0 = threadIdx.x - l0 * n;
      kstep = n;
    }
    if (l0 < lstep) {
      for (int k = k0; k < n; k += kstep) {
        const int q = signed_freq(k, n);
        const int aq = q < 0 ? -q : q;
        const R w = (2 * aq < n2_solve) ? R(1) : (2 * aq == n2_solve ? R(0.5) : R(0));
        const bool real_only = aq == 0 || 2 * aq == n2_solve;
        const int slot = L.blue ? sp(k) : sp(L.pos[k]);
        const cplx<R> ch = L.blue ? L.chirp[k] : mkc<R>(R(1), R(0));
        for (int line = l0; line < nlines; line += lstep) {
          const int rl = fdiv(line, g.dnp), p = line - rl * np;
          const long long row = row0 + rl;
          cplx<R> z = mkc<R>(R(0), R(0));
          if (row < nrows && w != R(0)) {
            const int ca = 2 * p, cb = 2 * p + 1;
            cplx<R> a = cscale<R>(spec_at(ca, rl, aq), w);
            cplx<R> bv = cb < C ? cscale<R>(spec_at(cb, rl, aq), w) : mkc<R>(R(0), R(0));
            if (real_only) { a.y = R(0); bv.y = R(0); }
            if (q < 0) { a.y = -a.y; bv.y = -bv.y; }     // X_{-k} = conj(X_k)
            z = mkc<R>(a.x - bv.y, a.y + bv.x);
          }
          buf[(long long)line * ld + slot] = L.blue ? cmul<R>(cconj<R>(z), ch) : z;
        }
      }
    }
  }
  zero_tail<R>(buf, ld, rows * np, L);
  __syncthreads();
  line_core<R>(buf, ld, rows * np, L, true);
  // 2) coefficient per voxel (all loads), in place, from the staged rows
  cp_async_wait<0>();
  __syncthreads();
  for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
    const int rl = fdiv(e, L.dn), j = e - rl * n;
    const long long row = row0 + rl;
    cplx<R>* base = buf + (long long)rl * np * ld;
    if (row >= nrows) {
      for (int p = 0; p < np; ++p) put_fwd<R>(base + p * ld, L, j, mkc<R>(R(0), R(0)));
      continue;
    }
    // slots of voxel j hold the inverse output; make them raw values first
    // (Bluestein outputs carry conj and chirp), then one load at a time: comp c
    // sits in pair line c/2 (real part for even c)
    if (L.blue) {
      for (int p = 0; p < np; ++p) {
        const cplx<R> z = get_inv<R>(base + p * ld, L, j);
        base[p * ld + sp(j)] = z;
      }
    }
    for (int l = 0; l < g.L; ++l) {
      R xv[kMaxDv], qv[kMaxDv];
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const int comp = l * g.dv + c;
        xv[c] = reinterpret_cast<const R*>(base + (comp >> 1) * ld + sp(j))[comp & 1];
      }
      if (st_coef) coef_apply<R, COEF>(acache, (long long)rows * n, (long long)rl * n + j, g.dv, xv, qv);
      else coef_apply<R, COEF>(A, Mi, row * n + j, g.dv, xv, qv);
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const int comp = l * g.dv + c;
        R* slot = reinterpret_cast<R*>(base + (comp >> 1) * ld + sp(j)) + (comp & 1);
        *slot = qv[c] * coef_scale;
      }
    }
    if (C & 1) reinterpret_cast<R*>(base + (np - 1) * ld + sp(j))[1] = R(0);
    if (L.blue) {  // forward Bluestein input carries the chirp
      for (int p = 0; p < np; ++p) {
        cplx<R>* slot = base + p * ld + sp(j);
        *slot = cmul<R>(*slot, L.chirp[j]);
      }
    }
  }
  __syncthreads();
  zero_tail<R>(buf, ld, rows * np, L);
  __syncthreads();
  line_core<R>(buf, ld, rows * np, L, false);
  // 3) split and keep the band (frequency-stationary as in 1)
  {
    int k0 = threadIdx.x, kstep = blockDim.x, l0 = 0, lstep = 1;
    if (n2h_band < (int)blockDim.x) {
      lstep = blockDim.x / n2h_band;
      l0 = threadIdx.x / n2h_band;
      k0 = threadIdx.x - l0 * n2h_band;
      kstep = n2h_band;
    }
    if (l0 < lstep) {
      for (int k = k0; k < n2h_band; k += kstep) {
        const bool keep = 2 * k <= n2_solve;
        const int km = k == 0 ? 0 : n - k;
        const int sk = L.blue ? sp(k) : sp(L.pos[k]);
        const int sm = L.blue ? sp(km) : sp(L.pos[km]);
        const cplx<R> chk = L.blue ? L.chirp[k] : mkc<R>(R(1), R(0));
        const cplx<R> chm = L.blue ? L.chirp[km] : mkc<R>(R(1), R(0));
        for (int line = l0; line < nlines; line += lstep) {
          const int rl = fdiv(line, g.dnp), p = line - rl * np;
          const long long row = row0 + rl;
          if (row >= nrows) continue;
          cplx<R> xa = mkc<R>(R(0), R(0)), xb = mkc<R>(R(0), R(0));
          if (keep) {
            const cplx<R>* lp = buf + (long long)line * ld;
            const cplx<R> zk = L.blue ? cmul<R>(lp[sk], chk) : lp[sk];
            const cplx<R> zm = L.blue ? cmul<R>(lp[sm], chm) : lp[sm];
            xa = mkc<R>(R(0.5) * (zk.x + zm.x), R(0.5) * (zk.y - zm.y));
            xb = mkc<R>(R(0.5) * (zk.y + zm.y), R(0.5) * (zm.x - zk.x));
            if (2 * k == n2_solve) { xa.y = R(0); xb.y = R(0); }  // mean of +-N/2 (real lines)
          }
          const int ca = 2 * p, cb = 2 * p + 1;
          S[((long long)ca * nrows + row) * n2h_band + k] = xa;
          if (cb < C) S[((long long)cb * nrows + row) * n2h_band + k] = xb;
        }
      }
    }
  }
}

// The isotropic middle of k_band_last_p2 in one pass over shared memory: the
// last inverse stage (S = 0, DIT), q = a(v) x / prod(N) per voxel, and the first
// forward stage (S = 0, DIF).  Both stages use the same butterflies, slots
// and twiddles, and after the inverse the slot j1 + q ms holds voxel j1 + q ms
// of the line, so the coefficient is applied in registers between them.
// Pair line p of row rl carries comps 2p, 2p+1, both scaled by a(v); the
// unused imaginary half of the last line (odd comp count) is zeroed, rows past
// the grid are zeroed, as in the unfused path.
template <typename R, int P, int K = 0>
__device__ __forceinline__ void p2_fused_iso_stage0(cplx<R>* __restrict__ buf, int ld, int nlines,
                                                    const cplx<R>* __restrict__ tw, int np,
                                                    FastDiv dnp, const R* acache,
                                                    const R* __restrict__ A, long long row0,
                                                    long long nrows, bool st_coef, R cs,
                                                    bool codd) {
  constexpr int E = p2_e(P, 0, K);
  constexpr int RAD = 1 << E;
  constexpr int LMS = P - E, MS = 1 << LMS, NBL = MS;
  constexpr int N = 1 << P;
  const int lstep = blockDim.x >> LMS;
  const int l0 = threadIdx.x >> LMS;
  const int j1 = threadIdx.x & (NBL - 1);
  const int sbase = sp(j1);
  cplx<R> w[RAD];
#pragma unroll
  for (int q = 1; q < RAD; ++q) w[q] = tw[j1 * q];
  for (int line = l0; line < nlines; line += lstep) {
    const int rl = fdiv(line, dnp), p = line - rl * np;
    const long long row = row0 + rl;
    const bool valid = row < nrows;
    const R* arow = st_coef ? acache + (long long)rl * N : A + (valid ? row : 0) * N;
    cplx<R>* lp = buf + line * ld + sbase;
    cplx<R> v[RAD];
    v[0] = cconj<R>(lp[0]);
#pragma unroll
    for (int q = 1; q < RAD; ++q) v[q] = cconj<R>(cmulc<R>(lp[sp(q * MS)], w[q]));
    dft_fwd<R, RAD>(v, tw, N);
    const bool zimag = codd && p == np - 1;
#pragma unroll
    for (int q = 0; q < RAD; ++q) {
      const cplx<R> x = cconj<R>(v[q]);
      if (valid) {
        const R a = arow[j1 + q * MS];
        v[q] = mkc<R>((a * x.x) * cs, zimag ? R(0) : (a * x.y) * cs);
      } else {
        v[q] = mkc<R>(R(0), R(0));
      }
    }
    dft_fwd<R, RAD>(v, tw, N);
    lp[0] = v[0];
#pragma unroll
    for (int q = 1; q < RAD; ++q) lp[sp(q * MS)] = cmul<R>(v[q], w[q]);
  }
}

// k_band_last for a direct power-of-two integration line B2 = 2^P (the
// smooth grids 2^k >= 2N-1 of the common solve sizes: 509 -> 512, 253 -> 256).
// Same shared-memory layout, staging and results as k_band_last; the phases
// around the transforms are organised per line instead of per element:
//  1) a warp expands one pair line: lane aq reads the two staged band spectra
//     once and writes frequency aq and its conjugate N-aq; the frequencies
//     outside the band get zeros.  Digit-reversed slots are shifts (p2_pos).
//  2) the coefficient per voxel; for isotropic coefficients both comps of a
//     pair line scale together (one 8- or 16-byte access per pair line).
//  3) a warp splits one pair line back into its two band half spectra with
//     coalesced stores.
template <typename R, int COEF, int P>
__global__ void __launch_bounds__(256, kFftMinBlocks<R>) k_band_last_p2(cplx<R>* __restrict__ S,
                                                   const R* __restrict__ A, const __grid_constant__ GridDims g,
                                                   long long nrows, int n2h_band, int n2_solve,
                                                   const __grid_constant__ LineDev<R> L, int rows, R coef_scale,
                                                   const int* __restrict__ all_done, int stage) {
  constexpr int N = 1 << P;
  // FP32 512-point lines run as 16 . 32 (p2_k_for), as the line plans do
  constexpr int K = p2_k_for<R>(P);
  if (all_done && *all_done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int C = g.L * g.dv;
  const int np = (C + 1) / 2;
  const int ld = L.ld;
  const long long Mi = nrows * N;
  const long long row0 = (long long)blockIdx.x * rows;
  const int cA = coef_comps<COEF>(g.dv);
  const int vrows = (int)((nrows - row0) < rows ? (nrows - row0) : rows);
  cplx<R>* sraw = reinterpret_cast<cplx<R>*>(
      smem_raw + align16((size_t)rows * np * ld * sizeof(cplx<R>)));
  R* acache = reinterpret_cast<R*>(
      reinterpret_cast<unsigned char*>(sraw) +
      ((stage & 1) ? align16((size_t)C * rows * n2h_band * sizeof(cplx<R>)) : 0));
  const bool st_spec = stage & 1, st_coef = stage & 2;
  if (st_spec)
    for (int c = 0; c < C; ++c)
      stage_async(sraw + (size_t)c * rows * n2h_band,
                  S + ((long long)c * nrows + row0) * n2h_band, vrows * n2h_band);
  cp_async_commit();
  if (st_coef)
    for (int t = 0; t < cA; ++t)
      stage_async(acache + (size_t)t * rows * N, A + (long long)t * Mi + row0 * N, vrows * N);
  cp_async_commit();
  cp_async_wait<1>();
  __syncthreads();
  const int nlines = rows * np;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  // the band |k| < n2h_band lies within N/4: the span-1 stages can skip the
  // zero digits (p2_stage PRUNE)
  const bool band4 = 4 * n2h_band <= N;
  // 1) Hermitian pair lines Z = A + iB
  for (int line = warp; line < nlines; line += nwarp) {
    const int rl = fdiv(line, g.dnp), p = line - rl * np;
    cplx<R>* lp = buf + (long long)line * ld;
    const bool valid = row0 + rl < nrows;
    const int ca = 2 * p, cb = 2 * p + 1;
    const cplx<R>* sa = st_spec ? sraw + ((size_t)ca * rows + rl) * n2h_band
                                : S + ((long long)ca * nrows + row0 + rl) * n2h_band;
    const cplx<R>* sb = st_spec ? sraw + ((size_t)cb * rows + rl) * n2h_band
                                : S + ((long long)cb * nrows + row0 + rl) * n2h_band;
    for (int aq = lane; aq < n2h_band; aq += 32) {
      cplx<R> a = mkc<R>(R(0), R(0)), b = mkc<R>(R(0), R(0));
      if (valid) {
        const R w = (2 * aq < n2_solve) ? R(1) : R(0.5);
        a = cscale<R>(sa[aq], w);
        if (cb < C) b = cscale<R>(sb[aq], w);
        if (aq == 0 || 2 * aq == n2_solve) { a.y = R(0); b.y = R(0); }
      }
      lp[sp(p2_pos<P, K>(aq))] = mkc<R>(a.x - b.y, a.y + b.x);
      if (aq > 0) lp[sp(p2_pos<P, K>(N - aq))] = mkc<R>(a.x + b.y, b.x - a.y);  // X_{-k} = conj(X_k)
    }
    // zeros outside the band.  With the band within N/4 the first inverse
    // stage reads the frequencies N/4 <= k < 3N/4 as zeros (pruned top
    // digits), so only [n2h, N/4) and [3N/4, N - n2h] are written.
    if (!band4) {
      for (int k = n2h_band + lane; k <= N - n2h_band; k += 32)
        lp[sp(p2_pos<P, K>(k))] = mkc<R>(R(0), R(0));
    } else {
      for (int k = n2h_band + lane; k < N / 4; k += 32)
        lp[sp(p2_pos<P, K>(k))] = mkc<R>(R(0), R(0));
      for (int k = 3 * (N / 4) + lane; k <= N - n2h_band; k += 32)
        lp[sp(p2_pos<P, K>(k))] = mkc<R>(R(0), R(0));
    }
  }
  __syncthreads();
  constexpr int NST = p2_nst(P, K);
  if constexpr (COEF == COEF_ISO) {
    // inverse stages NST-1 .. 1, fused stage 0 with the coefficient, forward
    // stages 1 .. NST-1; the span-1 stages pruned to the band when it fits N/4
    const bool codd = (C & 1) != 0;
    if (band4) p2_stage<R, P, NST - 1, true, true, K>(buf, ld, nlines, L.tw);
    else p2_stage<R, P, NST - 1, true, false, K>(buf, ld, nlines, L.tw);
    __syncthreads();
    if constexpr (NST > 2) { p2_stage<R, P, 1, true, false, K>(buf, ld, nlines, L.tw); __syncthreads(); }
    cp_async_wait<0>();
    __syncthreads();
    p2_fused_iso_stage0<R, P, K>(buf, ld, nlines, L.tw, np, g.dnp, acache, A, row0, nrows, st_coef,
                              coef_scale, codd);
    __syncthreads();
    if constexpr (NST > 2) { p2_stage<R, P, 1, false, false, K>(buf, ld, nlines, L.tw); __syncthreads(); }
    if (band4) p2_stage<R, P, NST - 1, false, true, K>(buf, ld, nlines, L.tw);
    else p2_stage<R, P, NST - 1, false, false, K>(buf, ld, nlines, L.tw);
    __syncthreads();
  } else {
    if (band4) {
      p2_stage<R, P, NST - 1, true, true, K>(buf, ld, nlines, L.tw);
      __syncthreads();
      if constexpr (NST > 2) { p2_stage<R, P, 1, true, false, K>(buf, ld, nlines, L.tw); __syncthreads(); }
      p2_stage<R, P, 0, true, false, K>(buf, ld, nlines, L.tw);
      __syncthreads();
    } else {
      p2_run<R, P, true, false, K>(buf, ld, nlines, L.tw);
    }
    // 2) coefficient per voxel (all loads), in place
    cp_async_wait<0>();
    __syncthreads();
    for (int e = threadIdx.x; e < (rows << P); e += blockDim.x) {
      const int rl = e >> P, j = e & (N - 1);
      const long long row = row0 + rl;
      cplx<R>* base = buf + (long long)rl * np * ld + sp(j);
      if (row >= nrows) {
        for (int p = 0; p < np; ++p) base[p * ld] = mkc<R>(R(0), R(0));
        continue;
      }
      if constexpr (COEF == COEF_ISO) {
        const R a = st_coef ? acache[(long long)rl * N + j] : A[row * N + j];
        for (int p = 0; p < np; ++p) {
          const cplx<R> z = base[p * ld];
          base[p * ld] = mkc<R>((a * z.x) * coef_scale, (a * z.y) * coef_scale);
        }
      } else {
        for (int l = 0; l < g.L; ++l) {
          R xv[kMaxDv], qv[kMaxDv];
  #pragma unroll
          for (int c = 0; c < kMaxDv; ++c) {
            if (c >= g.dv) break;
            const int comp = l * g.dv + c;
            xv[c] = reinterpret_cast<const R*>(base + (comp >> 1) * ld)[comp & 1];
          }
          if (st_coef) coef_apply<R, COEF>(acache, (long long)rows * N, (long long)rl * N + j, g.dv, xv, qv);
          else coef_apply<R, COEF>(A, Mi, row * N + j, g.dv, xv, qv);
  #pragma unroll
          for (int c = 0; c < kMaxDv; ++c) {
            if (c >= g.dv) break;
            const int comp = l * g.dv + c;
            reinterpret_cast<R*>(base + (comp >> 1) * ld)[comp & 1] = qv[c] * coef_scale;
          }
        }
      }
      if (C & 1) reinterpret_cast<R*>(base + (np - 1) * ld)[1] = R(0);
    }
    __syncthreads();
    if (band4) {
      p2_stage<R, P, 0, false, false, K>(buf, ld, nlines, L.tw);
      __syncthreads();
      if constexpr (NST > 2) { p2_stage<R, P, 1, false, false, K>(buf, ld, nlines, L.tw); __syncthreads(); }
      p2_stage<R, P, NST - 1, false, true, K>(buf, ld, nlines, L.tw);
      __syncthreads();
    } else {
      p2_run<R, P, false, false, K>(buf, ld, nlines, L.tw);
    }
  }
  // 3) split and keep the band
  for (int line = warp; line < nlines; line += nwarp) {
    const int rl = fdiv(line, g.dnp), p = line - rl * np;
    const long long row = row0 + rl;
    if (row >= nrows) continue;
    const cplx<R>* lp = buf + (long long)line * ld;
    const int ca = 2 * p, cb = 2 * p + 1;
    cplx<R>* da = S + ((long long)ca * nrows + row) * n2h_band;
    cplx<R>* db = S + ((long long)cb * nrows + row) * n2h_band;
    for (int k = lane; k < n2h_band; k += 32) {
      const cplx<R> zk = lp[sp(p2_pos<P, K>(k))];
      const cplx<R> zm = lp[sp(p2_pos<P, K>(k == 0 ? 0 : N - k))];
      cplx<R> xa = mkc<R>(R(0.5) * (zk.x + zm.x), R(0.5) * (zk.y - zm.y));
      cplx<R> xb = mkc<R>(R(0.5) * (zk.y + zm.y), R(0.5) * (zm.x - zk.x));
      if (2 * k == n2_solve) { xa.y = R(0); xb.y = R(0); }  // mean of +-N/2 (real lines)
      da[k] = xa;
      if (cb < C) db[k] = xb;
    }
  }
}

// ---------------------------------------------------------------------------
// Integration pass with register-resident 512-point lines (FP32, isotropic
// coefficient, band within a quarter of the line: the spheres configuration).
//
// One warp owns one pair line Z = X_a + i X_b at a time and keeps it in
// registers, 16 complex values per lane:
//  * frequency distribution: lane 2 k1 + h, register r holds Z[k1 + 16 h + 32 r]
//    (k1 < 16, h < 2, r < 16); the band |q| < n2h <= 128 lives in registers
//    0..3 and 12..15, the others are zero;
//  * space distribution: lane l, register j holds z[32 j + l].
// 512 = 16 x 32: a 16-point DFT in registers, the twiddles W512^(l k1), a
// transpose through a padded per-warp tile in shared memory, a radix-2 step
// between lane pairs (shuffles) and a second 16-point DFT in registers.
// Against the shared-memory cores each value crosses shared memory once per
// transform and no block barrier is needed.  The coefficient row lives in
// registers (lane l, register j: a[32 j + l]).
// ---------------------------------------------------------------------------
constexpr int kR512Warps = 8;            // warps per CTA
constexpr int kR512Tile = 16 * 34;       // transpose tile per warp (complex)

// tile slot of element (k1, l): rows of 34, the two lane halves 17 apart, so
// both transpose directions are free of bank conflicts
__device__ __forceinline__ int r512_slot(int k1, int l) { return 34 * k1 + 17 * (l >> 4) + (l & 15); }

// W32^r for r < 16 (compile-time after unrolling)
__device__ __forceinline__ float2 w32f(int r) {
  const float c[16] = {1.f, 0.98078528040323044912f, 0.92387953251128675613f, 0.83146961230254523708f,
                       0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                       0.19509032201612826785f, 0.f, -0.19509032201612826785f, -0.38268343236508977173f,
                       -0.55557023301960222474f, -0.70710678118654752440f, -0.83146961230254523708f,
                       -0.92387953251128675613f, -0.98078528040323044912f};
  const float sn[16] = {0.f, 0.19509032201612826785f, 0.38268343236508977173f, 0.55557023301960222474f,
                        0.70710678118654752440f, 0.83146961230254523708f, 0.92387953251128675613f,
                        0.98078528040323044912f, 1.f, 0.98078528040323044912f, 0.92387953251128675613f,
                        0.83146961230254523708f, 0.70710678118654752440f, 0.55557023301960222474f,
                        0.38268343236508977173f, 0.19509032201612826785f};
  return make_float2(c[r], -sn[r]);
}

// inverse transform of one pair line: frequency distribution in v, space
// distribution out (unnormalised)
__device__ __forceinline__ void r512_inverse(float2 (&v)[16], float2* tile, const float2* twt,
                                             int lane) {
  // 16-point inverse DFT over the registers (band: inputs 0..3, 12..15)
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r].y = -v[r].y;
  dft16<float, true>(v);
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r].y = -v[r].y;
  // odd lanes: times W32^(-l'), then the radix-2 step between lane pairs
  const bool odd = lane & 1;
  if (odd) {
#pragma unroll
    for (int r = 1; r < 16; ++r) v[r] = cmulc<float>(v[r], w32f(r));
  }
  const float sg = odd ? -1.f : 1.f;
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const float px = __shfl_xor_sync(0xffffffffu, v[r].x, 1);
    const float py = __shfl_xor_sync(0xffffffffu, v[r].y, 1);
    v[r] = make_float2(fmaf(sg, v[r].x, px), fmaf(sg, v[r].y, py));
  }
  // transpose: lane 2 k1 + g register l' holds Y[l' + 16 g][k1]
  const int k1 = lane >> 1, g = lane & 1;
#pragma unroll
  for (int r = 0; r < 16; ++r) tile[r512_slot(k1, r + 16 * g)] = v[r];
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = tile[r512_slot(r, lane)];
  __syncwarp();
  // W512^(-l k1), then the 16-point inverse DFT over k1
#pragma unroll
  for (int r = 1; r < 16; ++r) v[r] = cmulc<float>(v[r], twt[r * 32 + lane]);
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r].y = -v[r].y;
  dft16<float>(v);
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r].y = -v[r].y;
}

// forward transform: space distribution in v, frequency distribution out
// (registers 0..3 and 12..15 only: the band)
__device__ __forceinline__ void r512_forward(float2 (&v)[16], float2* tile, const float2* twt,
                                             int lane) {
  dft16<float>(v);
#pragma unroll
  for (int r = 1; r < 16; ++r) v[r] = cmul<float>(v[r], twt[r * 32 + lane]);
#pragma unroll
  for (int r = 0; r < 16; ++r) tile[r512_slot(r, lane)] = v[r];
  __syncwarp();
  const int k1 = lane >> 1, g = lane & 1;
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = tile[r512_slot(k1, r + 16 * g)];
  __syncwarp();
  const bool odd = lane & 1;
  const float sg = odd ? -1.f : 1.f;
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const float px = __shfl_xor_sync(0xffffffffu, v[r].x, 1);
    const float py = __shfl_xor_sync(0xffffffffu, v[r].y, 1);
    v[r] = make_float2(fmaf(sg, v[r].x, px), fmaf(sg, v[r].y, py));
  }
  if (odd) {
#pragma unroll
    for (int r = 1; r < 16; ++r) v[r] = cmul<float>(v[r], w32f(r));
  }
  dft16<float, false, true>(v);
}

// Per-warp shared memory of k_band_last_r512 (float2 units): the transpose
// tile, two staging buffers for a pair line's band spectra (2 x 128 complex
// each) and two for coefficient rows (512 floats each).
constexpr int kR512Stage = 2 * 128;
constexpr int kR512WarpSmem = kR512Tile + 2 * kR512Stage + 2 * 256;
// + two mbarriers per warp (the TMA path's stage buffers 0 and 1)
__host__ __device__ constexpr size_t r512_smem_bytes() {
  return (size_t)(16 * 32 + kR512Warps * kR512WarpSmem) * sizeof(float2) +
         (size_t)kR512Warps * 2 * sizeof(unsigned long long);
}
// tries of a bounded wait for a stage buffer (each try waits up to a
// hardware-chosen time): far beyond any copy, short of a hung launch
constexpr int kR512WaitTries = 1 << 22;

// S: band spectra [C][nrows][n2h] (in place); A: isotropic coefficient
// [nrows][512]; tw: W512^k, k < 512.  Requires n2h <= 128 and 2 n2h - 1 <=
// n2_solve + 1 (the band of the solve grid).  FULL: n2h = 128 and n2_solve =
// 255 (every band slot holds a frequency below the solve line's Nyquist: no
// per-frequency weights or tests).
// use_tma (FULL only): lane 0 of a warp loads the next pair line's spectra
// rows (tmS: S as [C * nrows][128] 8-byte elements) and coefficient row (tmA:
// A as [nrows][256] 8-byte elements) with TMA boxes that complete on the
// stage buffer's mbarrier, in place of per-lane cp.async.  A wait that runs
// out sets *err (and *stop, the CG's all-done flag, when given); the warp then
// waits (bounded) for its other copy and returns.  Each warp walks its pair lines
// (row by row, the np pair lines of a row in turn; with an odd component count
// two consecutive rows of the warp share the pair line of their last lines)
// and copies the next pair line's spectra (and, at a new row, the next
// coefficient row) into shared memory while it transforms the current one.  A template
// instantiated for float only, so the FP64 translation unit compiles none of it.
template <typename R, bool FULL>
__global__ void __launch_bounds__(32 * kR512Warps, 2) k_band_last_r512(
    float2* __restrict__ S, const float* __restrict__ A, const __grid_constant__ GridDims g,
    long long nrows, int n2h, int n2_solve, const float2* __restrict__ tw, float cs,
    const int* __restrict__ all_done, const __grid_constant__ CUtensorMap tmS,
    const __grid_constant__ CUtensorMap tmA, int use_tma, int* __restrict__ err,
    int* __restrict__ stop) {
  static_assert(sizeof(R) == 4, "FP32 lines");
  if (all_done && *all_done) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* twt = reinterpret_cast<float2*>(smem_raw);   // W512^(l k1) at [k1][l]
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(
      smem_raw + (size_t)(16 * 32 + kR512Warps * kR512WarpSmem) * sizeof(float2));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2* wsm = twt + 16 * 32 + warp * kR512WarpSmem;
  float2* tile = wsm;
  float2* stg = wsm + kR512Tile;                                            // [2][2][128]
  float* cst = reinterpret_cast<float*>(wsm + kR512Tile + 2 * kR512Stage);  // [2][512]
  unsigned long long* wbar = bars + 2 * warp;
  // TMA boxes land on 128-byte aligned stage buffers (checked, not assumed)
  const bool tma = FULL && use_tma &&
                   ((((unsigned)__cvta_generic_to_shared(stg)) | ((unsigned)__cvta_generic_to_shared(cst))) & 127u) == 0;
  if (tma && lane == 0) {
    mbar_init(wbar, 1);
    mbar_init(wbar + 1, 1);
    mbar_init_fence();
  }
  for (int e = threadIdx.x; e < 16 * 32; e += blockDim.x) twt[e] = tw[(e & 31) * (e >> 5)];
  __syncthreads();
  const int C = g.L * g.dv;
  const int np = (C + 1) / 2;
  const int k1 = lane >> 1, h = lane & 1;
  const int kl = k1 + 16 * h;
  const int plane = lane >= 2 ? 33 - lane : lane;   // lane of the frequency -k
  const long long gw = (long long)blockIdx.x * kR512Warps + warp;
  const long long nw = (long long)gridDim.x * kR512Warps;
  const long long nrow_w = gw < nrows ? (nrows - gw + nw - 1) / nw : 0;   // rows of this warp
  // An odd component count leaves one real line per row without a partner:
  // the warp's rows i and i + 1 (i even) put their last lines into one pair
  // line ("two"), X_a from row i and X_b from row i + 1, each multiplied by its
  // own coefficient row.  Tasks of such a row pair: row i's pair lines
  // 0..np-2, the shared line (its copy brings row i + 1's coefficient row),
  // row i + 1's pair lines 0..np-2; 2 np - 1 transforms for two rows instead
  // of 2 np.  A last unpaired row runs its np tasks alone.
  const bool comb = (C & 1) && np > 1;
  const long long T2 = 2 * np - 1;
  const long long npr = comb ? nrow_w / 2 : 0;
  const long long ntask = comb ? npr * T2 + (nrow_w & 1) * np : nrow_w * np;
  // Task position: block m (a row; with shared lines a row pair, then a last
  // unpaired row) and index u in it, advanced by one per task without integer
  // division.  place(): row index i of this warp (row gw + i nw), pair line p,
  // shared line.
  struct TaskPos {
    long long m;
    int u;
  };
  auto advance = [&](TaskPos& q) {
    const int lim = (comb && q.m < npr) ? (int)T2 : np;
    if (++q.u == lim) {
      q.u = 0;
      ++q.m;
    }
  };
  auto place = [&](const TaskPos& q, long long& i, int& p, bool& two) {
    if (comb && q.m < npr) {
      two = q.u == np - 1;
      i = q.u >= np ? 2 * q.m + 1 : 2 * q.m;
      p = q.u >= np ? q.u - np : q.u;
    } else {
      i = comb ? 2 * q.m : q.m;
      p = q.u;
      two = false;
    }
  };
  // copy task t into buffer t & 1; the coefficient row of row index i goes to
  // coefficient buffer i & 1 (the shared line brings row i + 1's)
  auto prefetch = [&](long long t, const TaskPos& q) {
    long long i = 0;
    int p = 0;
    bool two = false;
    if (t < ntask) place(q, i, p, two);
    const long long row = gw + i * nw;
    const int b = (int)(t & 1);
    const bool loadc = two || (p == 0 && !(comb && (i & 1)));
    const long long crow = two ? row + nw : row;
    float* cdst = cst + ((i + (two ? 1 : 0)) & 1) * 512;
    const int halves = (two || 2 * p + 1 < C) ? 2 : 1;
    // spectra row of half h: line 2p + h of this row, or line C - 1 of rows i, i + 1
    auto srow = [&](int half) {
      return two ? (long long)(C - 1) * nrows + row + half * nw
                 : (long long)(2 * p + half) * nrows + row;
    };
    if (tma) {
      if (t < ntask && lane == 0) {
        // the generic reads of these buffers (task t - 2) come first
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(wbar + b, (unsigned)(halves * 1024 + (loadc ? 2048 : 0)));
        for (int half = 0; half < halves; ++half)
          tma_load_2d(stg + (b * 2 + half) * 128, &tmS, 0, (int)srow(half), wbar + b);
        if (loadc) tma_load_2d(cdst, &tmA, 0, (int)crow, wbar + b);
      }
      return;
    }
    if (t < ntask) {
      for (int half = 0; half < halves; ++half) {
        const float2* src = S + srow(half) * n2h;
        float2* dst = stg + (b * 2 + half) * 128;
        for (int k = lane; k < n2h; k += 32) cp_async_small<8>(dst + k, src + k);
      }
      if (loadc) {
        const float* src = A + crow * 512;
        for (int j = lane; j < 128; j += 32) cp_async_16(cdst + 4 * j, src + 4 * j);
      }
    }
    cp_async_commit();
  };
  TaskPos cur{0, 0};
  prefetch(0, cur);
  float a[16];
  for (long long t = 0; t < ntask; ++t) {
    long long i;
    int p;
    bool two;
    place(cur, i, p, two);
    TaskPos nxt = cur;
    advance(nxt);
    const long long row = gw + i * nw;
    const int b = (int)(t & 1);
    __syncwarp();       // every lane is done with the buffers of task t - 1
    prefetch(t + 1, nxt);
    cur = nxt;
    if (tma) {
      if (!mbar_wait_bounded(wbar + b, (unsigned)((t >> 1) & 1), kR512WaitTries)) {
        if (lane == 0) {
          atomicExch(err, 1);
          if (stop) atomicExch(stop, 1);
        }
        // the other buffer's copies (task t + 1) before the warp leaves
        if (t + 1 < ntask)
          (void)mbar_wait_bounded(wbar + ((b + 1) & 1), (unsigned)(((t + 1) >> 1) & 1),
                                  kR512WaitTries);
        return;
      }
    } else {
      cp_async_wait<1>();
    }
    __syncwarp();       // task t's copies of every lane are visible
    if (p == 0 && !two) {
      const float* ar = cst + (i & 1) * 512;
#pragma unroll
      for (int j = 0; j < 16; ++j) a[j] = ar[32 * j + lane] * cs;
    }
    const int ca = 2 * p, cb = 2 * p + 1;
    const bool hb = two || cb < C;
    const float2* sa = stg + (b * 2) * 128;
    const float2* sb = stg + (b * 2 + 1) * 128;
    float2 v[16];
#pragma unroll
    for (int r = 4; r < 12; ++r) v[r] = make_float2(0.f, 0.f);
    // expand: Z_k = A_k + i B_k, Z_{-q} = conj(A_q) + i conj(B_q)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int k = kl + 32 * r;
      float2 za = make_float2(0.f, 0.f), zb = make_float2(0.f, 0.f);
      if constexpr (FULL) {
        // k < 128 = n2h and 2k < 255 = n2_solve for every lane
        za = sa[k];
        zb = hb ? sb[k] : make_float2(0.f, 0.f);
        if (r == 0 && kl == 0) { za.y = 0.f; zb.y = 0.f; }
      } else if (k < n2h) {
        const float w = (2 * k < n2_solve) ? 1.f : 0.5f;
        za = sa[k];
        zb = hb ? sb[k] : make_float2(0.f, 0.f);
        za.x *= w; za.y *= w; zb.x *= w; zb.y *= w;
        if (k == 0 || 2 * k == n2_solve) { za.y = 0.f; zb.y = 0.f; }
      }
      v[r] = make_float2(za.x - zb.y, za.y + zb.x);
      const int q = 512 - (kl + 32 * (15 - r));     // register 15 - r holds -q
      float2 ma = make_float2(0.f, 0.f), mb = make_float2(0.f, 0.f);
      if constexpr (FULL) {
        // q = 32 (r + 1) - kl: below 128 except q = 128 (r = 3, kl = 0)
        if (r < 3 || kl != 0) {
          ma = sa[q];
          mb = hb ? sb[q] : make_float2(0.f, 0.f);
        }
      } else if (q < n2h) {
        const float w = (2 * q < n2_solve) ? 1.f : 0.5f;
        ma = sa[q];
        mb = hb ? sb[q] : make_float2(0.f, 0.f);
        ma.x *= w; ma.y *= w; mb.x *= w; mb.y *= w;
        if (2 * q == n2_solve) { ma.y = 0.f; mb.y = 0.f; }
      }
      v[15 - r] = make_float2(ma.x + mb.y, mb.x - ma.y);
    }
    r512_inverse(v, tile, twt, lane);
    // q = a x cs on both real fields of the pair (the imaginary part is zero
    // when the line has no second field); the shared line takes row i's
    // coefficient (buffer 0, i even) on X_a and row i + 1's (buffer 1) on X_b
    if (two) {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        v[j] = make_float2((cst[32 * j + lane] * cs) * v[j].x,
                           (cst[512 + 32 * j + lane] * cs) * v[j].y);
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = make_float2(a[j] * v[j].x, hb ? a[j] * v[j].y : 0.f);
    }
    r512_forward(v, tile, twt, lane);
    // split: X_a = (Z_k + conj Z_-k) / 2, X_b = (Z_k - conj Z_-k) / 2i
    float2* da = S + (two ? (long long)(C - 1) * nrows + row : (long long)ca * nrows + row) * n2h;
    float2* db = S + (two ? (long long)(C - 1) * nrows + row + nw : (long long)cb * nrows + row) * n2h;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float mx = __shfl_sync(0xffffffffu, v[15 - r].x, plane);
      const float my = __shfl_sync(0xffffffffu, v[15 - r].y, plane);
      float2 zm = make_float2(mx, my);
      if (lane == 0) zm = v[(16 - r) & 15];   // k = 32 r: -k = 32 (16 - r)
      const int k = kl + 32 * r;
      if (FULL || k < n2h) {
        const float2 zk = v[r];
        float2 xa = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        float2 xb = make_float2(0.5f * (zk.y + zm.y), 0.5f * (zm.x - zk.x));
        if (!FULL && 2 * k == n2_solve) { xa.y = 0.f; xb.y = 0.f; }
        da[k] = xa;
        if (hb) db[k] = xb;
      }
    }
  }
  if (!tma) cp_async_wait<0>();
}

// W_i . u_j cross products per load pair on the solve grid (band energy):
// partial sums of sum_v sum_c W[i][c] (X[j][c] + delta_cj) (postprocess.py:53-70).
// LT = the plan's load count, so the per-thread sums are registers of fixed
// size and every value is loaded once: per voxel and component the L values
// of W and of X, then the L x L products.  Per-voxel products in the field
// precision, summed over 8 voxels, then into FP64 (FP64 arithmetic is the
// slow pipe on this GPU).  256 threads.
template <typename R, int LT>
__global__ void __launch_bounds__(256) k_cross_dot(const R* __restrict__ W, const R* __restrict__ X,
                                                   double* __restrict__ partials, GridDims g,
                                                   int add_macro) {
  __shared__ double red[8 * LT * LT];
  const int dv = g.dv;
  double acc[LT * LT];
  R part[LT * LT];
#pragma unroll
  for (int i = 0; i < LT * LT; ++i) {
    acc[i] = 0.;
    part[i] = R(0);
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  int cnt = 0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride) {
    for (int c = 0; c < dv; ++c) {
      R w[LT], x[LT];
#pragma unroll
      for (int i = 0; i < LT; ++i) {
        w[i] = W[(long long)(i * dv + c) * g.M + v];
        x[i] = X[(long long)(i * dv + c) * g.M + v] + ((add_macro && c == i) ? R(1) : R(0));
      }
#pragma unroll
      for (int i = 0; i < LT; ++i)
#pragma unroll
        for (int j = 0; j < LT; ++j) part[i * LT + j] += w[i] * x[j];
    }
    if (++cnt == 8) {
#pragma unroll
      for (int i = 0; i < LT * LT; ++i) {
        acc[i] += (double)part[i];
        part[i] = R(0);
      }
      cnt = 0;
    }
  }
#pragma unroll
  for (int i = 0; i < LT * LT; ++i) acc[i] += (double)part[i];
  block_sum_n(acc, LT * LT, red, partials + (long long)blockIdx.x * LT * LT);
}

// v E at frequency 0 of half spectra in the N layout [load][comp][n0][n1][n2h]
// (normalised, plain or z form: both are the mean there): comp l of load l
template <typename R>
__global__ void k_z_macro(cplx<R>* __restrict__ z, long long nzc, int L, int dv, double v) {
  const int l = threadIdx.x;
  if (l < L && l < dv) z[(long long)(l * dv + l) * nzc].x += (R)v;
}

// x + E (macroscopic field added per load), for the band energy
template <typename R>
__global__ void k_add_macro(const R* __restrict__ X, R* __restrict__ U, GridDims g) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tot = (long long)g.L * g.dv * g.M;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    const long long comp = i / g.M;
    const int l = (int)(comp / g.dv), c = (int)(comp - (long long)l * g.dv);
    U[i] = X[i] + ((c == l) ? R(1) : R(0));
  }
}


// r = b - ax ; partial sum r^2 per load
template <typename R>
__global__ void __launch_bounds__(256) k_residual(const R* __restrict__ b, const R* __restrict__ ax,
                                                  R* __restrict__ r, double* __restrict__ partials,
                                                  GridDims g) {
  {  // the cell of a batched plan (grid y)
    const long long k = blockIdx.y;
    b += k * g.sf;
    ax += k * g.sf;
    r += k * g.sf;
    partials += k * gridDim.x * g.L;
  }
  __shared__ double red[8 * kMaxLoads];
  double acc[kMaxLoads];
  for (int i = 0; i < kMaxLoads; ++i) acc[i] = 0.;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M; v += stride)
    for (int l = 0; l < g.L; ++l)
      for (int c = 0; c < g.dv; ++c) {
        const long long i = (long long)(l * g.dv + c) * g.M + v;
        const R rv = b[i] - ax[i];
        r[i] = rv;
        acc[l] += (double)rv * (double)rv;
      }
  block_sum_n(acc, g.L, red, partials + (long long)blockIdx.x * g.L);
}

// dst = s_j * src, src in FP64, s one scale per load of every cell (device,
// cells x loads; refinement: scaled residual into the working precision)
template <typename RO>
__global__ void k_scale_from64(const double* __restrict__ src, RO* __restrict__ dst, long long tot,
                               long long per, const double* __restrict__ s) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride)
    dst[i] = (RO)(s[i / per] * src[i]);
}

// x += s_j * d, x in FP64 (refinement: correction of the working precision)
template <typename RI>
__global__ void k_add_scaled_to64(const RI* __restrict__ d, double* __restrict__ x, long long tot,
                                  long long per, const double* __restrict__ s) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride)
    x[i] += s[i / per] * (double)d[i];
}

// precision conversion
template <typename RO, typename RI>
__global__ void k_convert(long long n, const RI* __restrict__ in, RO* __restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (RO)in[i];
}

// ---------------------------------------------------------------------------
// Potential formulation (ffthompy/tensorsLowRank/homogenisation.py:41-127).
// The unknown is a scalar potential in the 'r' Fourier form of the grid N
// (unnormalised half spectrum [load][n0][n1][n2/2+1]); the operator is
//   P (-div) decrease_N F_Ns A iF_Ns enlarge_Ns grad P,
// P = 1/|2 pi xi| (1 at the mean), Ns = N (GaNi) or 2N-1 (Ga; N odd).
// Inside CG the iterates are held as z = sqrt(w) x / prod(N) with w the
// weight of the 'r' inner product (objects.py:618-631: 1 on the k2 = 0 and
// even-N Nyquist planes, 2 elsewhere), so that the reference's inner product
// is the Euclidean one of z and the generic CG kernels apply.
// ---------------------------------------------------------------------------
struct PotParams {
  int nb[3];       // potential grid N (GridDims axis order; nb[0] = 1 in 2D)
  int nbh;         // nb[2] / 2 + 1
  double Yg[3];    // cell size per GridDims axis
  double scale;    // enlargement prod(Ns)/prod(N)
  double zs;       // 1 / prod(N)
  // the per-launch factors, formed on the host (an FP64 division per thread
  // runs on the slow FP64 pipe): 2 pi / Yg, 1 / zs, 1 / scale, in both precisions
  double tpy[3], izs, iscale;
  float tpy_f[3], scale_f, zs_f, izs_f, iscale_f;
};

template <typename R>
__device__ __forceinline__ R pot_pick(float f, double d) {
  if constexpr (sizeof(R) == 4) return f; else return d;
}

// frequency of index k on an n-point axis in the reference's 'r' form
// (trigpol.py:27-40): 0..ceil(n/2)-1, then negative; the even-n Nyquist
// index carries -n/2, also on the half axis
__device__ __forceinline__ int ref_freq(int k, int n) { return k < (n + 1) / 2 ? k : k - n; }


// 2 pi xi per axis and P at frequency q in the field precision T (dim 2:
// q[0] = 0); tpy = 2 pi / Y per axis
template <typename T>
__device__ __forceinline__ T pot_symbols_t(int dim, const int* q, const T* tpy, T* tpx) {
  T k2 = T(0);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tpx[a] = (a == 0 && dim == 2) ? T(0) : tpy[a] * (T)q[a];
    k2 += tpx[a] * tpx[a];
  }
  return (q[0] == 0 && q[1] == 0 && q[2] == 0) ? T(1) : T(1) / sqrt(k2);
}

// S[l*d + a] (solve grid half spectrum) = scale * 2 pi i xi_a * P * x_l on the
// band of N, 0 elsewhere; x natural (zin = 0) or z-scaled (zin = 1).  Grid y
// is the load; the symbols are evaluated in the field precision.
template <typename R>
__global__ void k_pot_expand(const cplx<R>* __restrict__ xin, cplx<R>* __restrict__ S,
                             const __grid_constant__ GridDims g,
                             const __grid_constant__ PotParams pp, int zin,
                             const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const int Ms = g.n0 * g.n1 * g.n2h;
  const long long Mn = (long long)pp.nb[0] * pp.nb[1] * pp.nbh;
  const int d = g.dim;
  const int l = blockIdx.y;
  R tpy[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) tpy[a] = pot_pick<R>(pp.tpy_f[a], pp.tpy[a]);
  const R fs = pot_pick<R>(pp.scale_f, pp.scale);
  const R fz = pot_pick<R>(pp.izs_f, pp.izs);
  const cplx<R>* xl = xin + (long long)l * Mn;
  cplx<R>* Sl = S + (long long)(l * d) * Ms;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < Ms; v += gridDim.x * blockDim.x) {
    const int r = fdiv(v, g.dn2h);
    const int i2 = v - r * g.n2h;
    const int i0 = r / g.n1, i1 = r - i0 * g.n1;
    const int q[3] = {ref_freq(i0, g.n0), ref_freq(i1, g.n1), ref_freq(i2, g.n2)};
    const int ns[3] = {g.n0, g.n1, g.n2};
    bool in = true;
    int kn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int n = pp.nb[a];
      if (ns[a] != n) in = in && (2 * (q[a] < 0 ? -q[a] : q[a]) < n);
      kn[a] = q[a] >= 0 ? q[a] : q[a] + n;
    }
    cplx<R>* out = Sl + v;
    if (!in) {
      for (int a = 0; a < d; ++a) out[(long long)a * Ms] = mkc<R>(R(0), R(0));
      continue;
    }
    const cplx<R> u0 = xl[((long long)kn[0] * pp.nb[1] + kn[1]) * pp.nbh + kn[2]];
    R tpx[3];
    R f = pot_symbols_t<R>(d, q, tpy, tpx) * fs;
    // z form: divide by zs sqrt(w), w = 1 on k2 = 0 and the even Nyquist, else 2
    if (zin) f *= fz * ((kn[2] == 0 || 2 * kn[2] == pp.nb[2]) ? R(1) : R(0.70710678118654752440));
    const R ux = u0.x * f, uy = u0.y * f;
    for (int a = 0; a < d; ++a) {
      const R t = tpx[3 - d + a];
      out[(long long)a * Ms] = mkc<R>(-t * uy, t * ux);
    }
  }
}

// y_l (potential grid half spectrum) = sign * P / scale * sum_a 2 pi i xi_a
// S[l*d + a] read at the band frequencies of the solve grid; y natural
// (zout = 0) or z-scaled (zout = 1).  Grid y is the load.
template <typename R>
__global__ void k_pot_contract(const cplx<R>* __restrict__ S, cplx<R>* __restrict__ y,
                               const __grid_constant__ GridDims g,
                               const __grid_constant__ PotParams pp, double sign, int zout,
                               const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const long long Ms = (long long)g.n0 * g.n1 * g.n2h;
  const int Mn = pp.nb[0] * pp.nb[1] * pp.nbh;
  const int d = g.dim;
  const int l = blockIdx.y;
  R tpy[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) tpy[a] = pot_pick<R>(pp.tpy_f[a], pp.tpy[a]);
  const R fs = pot_pick<R>(pp.iscale_f, pp.iscale) * (sign < 0 ? R(-1) : R(1));
  const R fz = pot_pick<R>(pp.zs_f, pp.zs);
  const cplx<R>* Sl = S + (long long)(l * d) * Ms;
  cplx<R>* yl = y + (long long)l * Mn;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < Mn; v += gridDim.x * blockDim.x) {
    const int r = v / pp.nbh;
    const int k2 = v - r * pp.nbh;
    const int k0 = r / pp.nb[1], k1 = r - k0 * pp.nb[1];
    const int q[3] = {ref_freq(k0, pp.nb[0]), ref_freq(k1, pp.nb[1]), ref_freq(k2, pp.nb[2])};
    const int ns[3] = {g.n0, g.n1, g.n2};
    int ks[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) ks[a] = q[a] >= 0 ? q[a] : q[a] + ns[a];
    const long long sv = ((long long)ks[0] * g.n1 + ks[1]) * g.n2h + ks[2];
    R tpx[3];
    R f = pot_symbols_t<R>(d, q, tpy, tpx) * fs;
    if (zout) f *= fz * ((k2 == 0 || 2 * k2 == pp.nb[2]) ? R(1) : R(1.4142135623730950488));
    R ax = R(0), ay = R(0);
    for (int a = 0; a < d; ++a) {
      const cplx<R> sa = Sl[(long long)a * Ms + sv];
      const R t = tpx[3 - d + a];
      ax -= t * sa.y;
      ay += t * sa.x;
    }
    yl[v] = mkc<R>(f * ax, f * ay);
  }
}

// natural <-> z scaling of potential spectra (to_z: z = zs sqrt(w) x; w = 1
// on k2 = 0 and the even Nyquist, else 2)
template <typename R>
__global__ void k_pot_zscale(const cplx<R>* __restrict__ in, cplx<R>* __restrict__ out,
                             long long tot, const __grid_constant__ PotParams pp, int to_z) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const R zs = pot_pick<R>(pp.zs_f, pp.zs), izs = pot_pick<R>(pp.izs_f, pp.izs);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += stride) {
    const int k2 = (int)(e % pp.nbh);
    const bool one = k2 == 0 || 2 * k2 == pp.nb[2];
    const R f = to_z ? zs * (one ? R(1) : R(1.4142135623730950488))
                     : izs * (one ? R(1) : R(0.70710678118654752440));
    const cplx<R> u = in[e];
    out[e] = mkc<R>(f * u.x, f * u.y);
  }
}

// P = R + beta P for the active loads (solver.py:131)
template <typename R>
__global__ void k_p_update(const R* __restrict__ r, R* __restrict__ p, GridDims g,
                           const LoadState* __restrict__ st, const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const long long per = (long long)g.dv * g.M;
  const long long tot = (long long)g.L * per;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += stride) {
    const int l = (int)(i / per);
    if (st[l].done) continue;
    p[i] = r[i] + (R)st[l].beta * p[i];
  }
}

// ---------------------------------------------------------------------------
// Richardson, Chebyshev and BiCG recurrences over the fused operator
// (ffthompy/general/solver.py:63-77, 142-285), one component row per CTA row
// (grid (x, L*dv)) with partial sums in the layout of k_cg_update_comp.
// Loads whose state is done are left untouched.
// ---------------------------------------------------------------------------
// MODE 0 (Richardson): x += omega (b - ax), partial |b - ax|^2;
// MODE 1 (Chebyshev residual): r = b - ax, partial |r|^2.
template <typename R, int MODE>
__global__ void __launch_bounds__(256) k_resid_comp(const R* __restrict__ b,
                                                    const R* __restrict__ ax,
                                                    R* __restrict__ out, double omega,
                                                    double* __restrict__ partials, GridDims g,
                                                    const LoadState* __restrict__ st,
                                                    const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8];
  const int comp = blockIdx.y;
  const int l = comp / g.dv;
  double acc = 0.;
  if (!st[l].done) {
    const long long off = (long long)comp * g.M;
    const R w = (R)omega;
    R sq = R(0);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M;
         v += (long long)gridDim.x * blockDim.x) {
      const R r = b[off + v] - ax[off + v];
      if (MODE == 0) out[off + v] = out[off + v] + w * r;
      else out[off + v] = r;
      sq += r * r;
    }
    acc = (double)sq;
  }
  double t = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    double* o = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L;
    for (int k = 0; k < g.L; ++k) o[k] = k == l ? tot : 0.;
  }
}

// Chebyshev two-term coefficients of the iteration about to run (its number
// k = kit + 1), per active load: k = 1: p = 0, w = 1/d; k = 2: p = -(c/d)^2/2,
// w = 1/(d - c^2/(2d)); then p = -(c^2/4) w^2, w = 1/(d - c^2 w/4) with the
// previous w (solver.py:250-262).  p -> beta, w -> alpha.
static __global__ void k_cheb_coef(LoadState* st, int L, double d, double c,
                                   const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const int l = threadIdx.x;
  if (l >= L || st[l].done) return;
  const int k = st[l].kit + 1;
  double p, w;
  if (k == 1) {
    p = 0.;
    w = 1. / d;
  } else if (k == 2) {
    p = -(1. / 2.) * (c / d) * (c / d);
    w = 1. / (d - c * c / 2. / d);
  } else {
    const double wp = st[l].alpha;
    p = -(c * c / 4.) * wp * wp;
    w = 1. / (d - c * c * wp / 4.);
  }
  st[l].beta = p;
  st[l].alpha = w;
}

// norm_res of every load set to v (Richardson starts from 1e15, solver.py:65-66)
static __global__ void k_set_norm(LoadState* st, int L, double v) {
  const int l = threadIdx.x;
  if (l < L) st[l].norm_res = v;
}

// Chebyshev start (solver.py:226-236): r0 = sqrt(<r,r>), kept in pap; norm_res
// = r0 / sqrt(<B,B>); stop at once if norm_res < tol.  rpart: partials of
// k_resid_comp (nr parts), bpart: of k_dot (nb parts).
static __global__ void k_cheb_init(const double* __restrict__ rpart, int nr,
                                   const double* __restrict__ bpart, int nb, LoadState* st, int L,
                                   double invM, double* __restrict__ res_log, int log_cap) {
  const int l = threadIdx.x;
  if (l >= L) return;
  double sr = 0., sb = 0.;
  for (int i = 0; i < nr; ++i) sr += rpart[(long long)i * L + l];
  for (int i = 0; i < nb; ++i) sb += bpart[(long long)i * L + l];
  LoadState& S = st[l];
  const double r0 = sqrt(sr * invM);
  S.pap = r0;
  S.norm_res = (1.0 / sqrt(sb * invM)) * r0;
  S.kit = 0;
  S.alpha = 0.;
  S.beta = 0.;
  S.status = isfinite(S.norm_res) ? 0 : 3;
  S.done = !(S.norm_res > S.tol && S.maxiter > 0) || S.status != 0;
  if (res_log && log_cap > 0) res_log[l] = S.norm_res;
}

// Chebyshev update: v = r - p v, x += w v
template <typename R>
__global__ void __launch_bounds__(256) k_cheb_update(const R* __restrict__ r, R* __restrict__ v,
                                                     R* __restrict__ x, GridDims g,
                                                     const LoadState* __restrict__ st,
                                                     const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const int comp = blockIdx.y;
  const int l = comp / g.dv;
  if (st[l].done) return;
  const R p = (R)st[l].beta, w = (R)st[l].alpha;
  const long long off = (long long)comp * g.M;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g.M;
       i += (long long)gridDim.x * blockDim.x) {
    const R vn = r[off + i] - p * v[off + i];
    v[off + i] = vn;
    x[off + i] = x[off + i] + w * vn;
  }
}

// Residual norms of Richardson / Chebyshev: norm = sqrt(sum / M) * scale_l
// (scale: 1, or 1 / r0 held in pap for Chebyshev), kit + 1, the residual log
// and the stopping test norm > tol && kit < maxiter (solver.py:70-76, 263-281).
static __global__ void k_fin_norm(const double* __restrict__ partials, int nparts, LoadState* st,
                                  int L, double invM, int relative, double* __restrict__ res_log,
                                  int log_cap, int* all_done) {
  __shared__ double red[8];
  const int l = blockIdx.x;
  if (*all_done || st[l].done) return;
  double s = 0.;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(long long)i * L + l];
  double t = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    LoadState& S = st[l];
    S.kit += 1;
    double nrm = sqrt(tot * invM);
    if (relative) nrm = (1.0 / S.pap) * nrm;
    S.norm_res = nrm;
    if (res_log && S.kit < log_cap) res_log[(long long)S.kit * L + l] = nrm;
    if (!isfinite(nrm)) { S.status = 3; S.done = 1; }
    if (!(nrm > S.tol && S.kit < S.maxiter)) S.done = 1;
  }
}

// BiCG update: x += alpha P, R -= alpha AP, Rs -= alpha AT Ps, partial <R, Rs>
template <typename R>
__global__ void __launch_bounds__(256) k_bicg_update(R* __restrict__ x, R* __restrict__ r,
                                                     R* __restrict__ rs, const R* __restrict__ p,
                                                     const R* __restrict__ ap,
                                                     const R* __restrict__ atps,
                                                     double* __restrict__ partials, GridDims g,
                                                     const LoadState* __restrict__ st,
                                                     const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8];
  const int comp = blockIdx.y;
  const int l = comp / g.dv;
  double acc = 0.;
  if (!st[l].done) {
    const R a = (R)st[l].alpha;
    const long long off = (long long)comp * g.M;
    R sq = R(0);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.M;
         v += (long long)gridDim.x * blockDim.x) {
      const long long i = off + v;
      x[i] = x[i] + a * p[i];
      const R rn = r[i] - a * ap[i];
      const R sn = rs[i] - a * atps[i];
      r[i] = rn;
      rs[i] = sn;
      sq += rn * sn;
    }
    acc = (double)sq;
  }
  double t = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    double* o = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L;
    for (int k = 0; k < g.L; ++k) o[k] = k == l ? tot : 0.;
  }
}

// BiCG directions: P = R + beta P, Ps = Rs + beta Ps
template <typename R>
__global__ void __launch_bounds__(256) k_bicg_dirs(const R* __restrict__ r,
                                                   const R* __restrict__ rs, R* __restrict__ p,
                                                   R* __restrict__ ps, GridDims g,
                                                   const LoadState* __restrict__ st,
                                                   const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  const int comp = blockIdx.y;
  const int l = comp / g.dv;
  if (st[l].done) return;
  const R be = (R)st[l].beta;
  const long long off = (long long)comp * g.M;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g.M;
       i += (long long)gridDim.x * blockDim.x) {
    p[off + i] = r[off + i] + be * p[off + i];
    ps[off + i] = rs[off + i] + be * ps[off + i];
  }
}

// Spectral CG iterates of band plans: half spectra V (N layout
// [C][n0][n1][n2h]) and their z form z = sqrt(w) V f (to_z) or V = z f /
// sqrt(w) (from z), w the half-spectrum weight of the last-axis frequency.
template <typename R>
__global__ void k_half_weight(const cplx<R>* __restrict__ in, cplx<R>* __restrict__ out,
                              long long tot, int n2h, int n2, double f, int to_z) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const R fr = (R)f;   // the field precision per element (FP64 is the slow pipe)
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += stride) {
    const int k2 = (int)(e % n2h);
    const bool single = k2 == 0 || 2 * k2 == n2;
    const R fw = single ? fr : fr * (to_z ? R(1.4142135623730950488016887242097)
                                          : R(0.70710678118654752440084436210485));
    const cplx<R> u = in[e];
    out[e] = mkc<R>(fw * u.x, fw * u.y);
  }
}

// z <- G(xi) z at every frequency of half spectra in the N layout, all loads
// x += alpha p ; r -= alpha G(Ap) on the spectral iterates (z form, half
// spectra of the solve grid [load][comp][n0][n1][n2h]), partial <r, r> per
// CTA and load (grid y = load).  Ap arrives from the last axis pass without
// G: p lies in range(G) and G is self-adjoint, so <p, Ap> = <p, G Ap> was
// taken there, and G maps Ap onto range(G) here, where r stays
// (ffthompy/general/solver.py:127-129 with the operator's final projection
// moved into the update; gp.scale 1: the orthogonal projection).
template <typename R, int PHYS>
__global__ void __launch_bounds__(256) k_cg_update_spec(cplx<R>* __restrict__ x,
                                                        cplx<R>* __restrict__ r,
                                                        const cplx<R>* __restrict__ p,
                                                        const cplx<R>* __restrict__ ap,
                                                        double* __restrict__ partials,
                                                        const __grid_constant__ GridDims g,
                                                        const __grid_constant__ GreenParams gp,
                                                        FastDiv dn1,
                                                        const LoadState* __restrict__ st,
                                                        const int* __restrict__ all_done) {
  if (all_done && *all_done) return;
  __shared__ double red[8];
  const int l = blockIdx.y;
  const int F = g.n0 * g.n1 * g.n2h;
  double acc = 0.;
  if (!st[l].done) {
    const R a = (R)st[l].alpha;
    R part = R(0);   // up to 8 frequencies in the field precision, then FP64
    int cnt = 0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < F; f += gridDim.x * blockDim.x) {
      const int q = fdiv(f, g.dn2h);
      const int k2 = f - q * g.n2h;
      const int i0 = fdiv(q, dn1), i1 = q - i0 * g.n1;
      int kv[3];
      if (g.dim == 3) {
        kv[0] = signed_freq(i0, g.n0);
        kv[1] = signed_freq(i1, g.n1);
        kv[2] = k2;
      } else {
        kv[0] = signed_freq(i1, g.n1);
        kv[1] = k2;
      }
      cplx<R> v[kMaxDv];
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c)
        if (c < g.dv) v[c] = ap[(long long)(l * g.dv + c) * F + f];
      green_apply<R, PHYS>(gp, g.dim, kv, v);
#pragma unroll
      for (int c = 0; c < kMaxDv; ++c) {
        if (c >= g.dv) break;
        const long long i = (long long)(l * g.dv + c) * F + f;
        const cplx<R> pc = p[i], xc = x[i], rc = r[i];
        x[i] = mkc<R>(xc.x + a * pc.x, xc.y + a * pc.y);
        const cplx<R> rn = mkc<R>(rc.x - a * v[c].x, rc.y - a * v[c].y);
        r[i] = rn;
        part += rn.x * rn.x + rn.y * rn.y;
      }
      if (++cnt == 8) {
        acc += (double)part;
        part = R(0);
        cnt = 0;
      }
    }
    acc += (double)part;
  }
  const double t = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    double* out = partials + ((long long)blockIdx.y * gridDim.x + blockIdx.x) * g.L;
    for (int k = 0; k < g.L; ++k) out[k] = k == l ? tot : 0.;
  }
}

// (the orthogonal projection: gp.scale 1; zero outside the band)
template <typename R, int PHYS>
__global__ void k_spec_green(cplx<R>* __restrict__ z, GridDims g, GreenParams gp) {
  const long long F = (long long)g.n0 * g.n1 * g.n2h;
  const long long tot = (long long)g.L * F;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += stride) {
    const int l = (int)(e / F);
    const long long f = e - (long long)l * F;
    const int k2 = (int)(f % g.n2h);
    const long long r = f / g.n2h;
    const int i1 = (int)(r % g.n1), i0 = (int)(r / g.n1);
    int kv[3];
    if (g.dim == 3) {
      kv[0] = signed_freq(i0, g.n0);
      kv[1] = signed_freq(i1, g.n1);
      kv[2] = k2;
    } else {
      kv[0] = signed_freq(i1, g.n1);
      kv[1] = k2;
    }
    cplx<R> x[kMaxDv];
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < g.dv) x[c] = z[((long long)l * g.dv + c) * F + f];
    green_apply<R, PHYS>(gp, g.dim, kv, x);
#pragma unroll
    for (int c = 0; c < kMaxDv; ++c)
      if (c < g.dv) z[((long long)l * g.dv + c) * F + f] = x[c];
  }
}

}  // namespace fhp
