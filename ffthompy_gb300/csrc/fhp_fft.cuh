// Shared-memory line FFTs for the Fourier-Galerkin operator (sm_103a).
//
// A "line" is one 1D transform of logical length n held in shared memory.
//  * direct lines: n factors into radices {2,4,8,16} and the odd primes
//    3, 5, 7, 11, 13, 17;
//    forward = in-place decimation-in-frequency (natural in, digit-reversed
//    out), inverse = in-place decimation-in-time (digit-reversed in, natural
//    out).  No ping-pong buffer is needed: every butterfly reads and writes
//    the same r slots.
//  * Bluestein lines: n has a prime factor > 17 (19, 89, 127, 509, 1021 ...);
//    the DFT is a chirp convolution of smooth length m >= 2n-1 done with the
//    direct machinery (DIF, pointwise product with the filter spectrum stored
//    in digit-reversed order, DIT).
// Callers put/get values in *frequency* order through put_inv/get_fwd, so the
// permutation never leaves shared memory and global spectra stay in natural
// order (the layout of numpy's rfftn, ffthompy/tensors/fft.py:39-43).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fhp {

template <typename R> struct CplxT;
template <> struct CplxT<float> { using T = float2; };
template <> struct CplxT<double> { using T = double2; };
template <typename R> using cplx = typename CplxT<R>::T;

template <typename R>
__host__ __device__ __forceinline__ cplx<R> mkc(R a, R b) { cplx<R> c; c.x = a; c.y = b; return c; }
template <typename R>
__device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) { return mkc<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) { return mkc<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return mkc<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename R>
__device__ __forceinline__ cplx<R> cmulc(cplx<R> a, cplx<R> b) {
  return mkc<R>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename R>
__device__ __forceinline__ cplx<R> cconj(cplx<R> a) { return mkc<R>(a.x, -a.y); }
template <typename R>
__device__ __forceinline__ cplx<R> cscale(cplx<R> a, R s) { return mkc<R>(a.x * s, a.y * s); }
// -i * a
template <typename R>
__device__ __forceinline__ cplx<R> cmul_mi(cplx<R> a) { return mkc<R>(a.y, -a.x); }
// +i * a
template <typename R>
__device__ __forceinline__ cplx<R> cmul_pi(cplx<R> a) { return mkc<R>(-a.y, a.x); }

constexpr int kMaxStages = 16;
// power-of-two core lengths 2^kP2Min .. 2^kP2Max run compile-time stages
constexpr int kP2Min = 5;
constexpr int kP2Max = 10;

// Division by a run-time invariant d as a multiply-high and two shifts
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, round-up variant): exact for every 32-bit x.
struct FastDiv {
  unsigned m;
  unsigned char s1, s2;
  unsigned short pad;
};
inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f{};
  int l = 0;
  while ((1ull << l) < d) ++l;
  f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  f.s1 = (unsigned char)(l < 1 ? l : 1);
  f.s2 = (unsigned char)(l > 1 ? l - 1 : 0);
  return f;
}
__host__ __device__ __forceinline__ int fdiv(int x, FastDiv f) {
#ifdef __CUDA_ARCH__
  const unsigned t = __umulhi((unsigned)x, f.m);
#else
  const unsigned t = (unsigned)(((unsigned long long)(unsigned)x * f.m) >> 32);
#endif
  return (int)((t + (((unsigned)x - t) >> f.s1)) >> f.s2);
}

// Padded shared-memory slot of line element i: one spare slot per 32 elements
// breaks the power-of-two strides of the late radix stages across banks.
__device__ __forceinline__ int sp(int i) { return i + (i >> 5); }
__host__ __device__ inline int padded_ld(int nf) { return nf + (nf >> 5) + 1; }
__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// ---------------------------------------------------------------------------
// Asynchronous global -> shared staging (cp.async, LDGSTS): copies go straight
// to shared memory without registers, so a thread can keep many in flight
// (the load phases are latency-bound otherwise).  Completion is waited for in
// hardware (cp.async.wait_group), with no spin loop.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <int BYTES>
__device__ __forceinline__ void cp_async_small(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------------------
// Tensor-memory-access (TMA) tile loads completing on an mbarrier: one thread
// issues a 2D box copy global -> shared, the barrier counts the bytes, and the
// consumers wait on the barrier's phase with a bounded number of tries.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
// the barrier initialisation is visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// generic-proxy accesses of shared memory are ordered before later async copies
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes)
               : "memory");
}
// one try: 1 once the phase of the given parity has completed
__device__ __forceinline__ unsigned mbar_try_wait(unsigned long long* bar, unsigned parity) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok;
}
// bounded wait: false when the phase has not completed after `tries` tries
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  int tries) {
  for (int i = 0; i < tries; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// 2D box (x innermost, in elements) of the tensor map tm into shared memory
__device__ __forceinline__ void tma_load_2d(void* smem, const void* tm, int x, int y,
                                            unsigned long long* bar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(d),
      "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(b)
      : "memory");
}

// Block-cooperative copy of count elements of T (4, 8 or 16 bytes) from global
// to shared memory: 16-byte copies when both ends are 16-byte aligned and the
// length is a multiple of 16 bytes, element copies otherwise.
template <typename T>
__device__ __forceinline__ void stage_async(T* dst, const T* src, int count) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "element size");
  const size_t bytes = (size_t)count * sizeof(T);
  const bool vec = (((size_t)__cvta_generic_to_shared(dst) | reinterpret_cast<size_t>(src) |
                     bytes) & 15) == 0;
  if (vec) {
    const int n16 = (int)(bytes >> 4);
    char* d = reinterpret_cast<char*>(dst);
    const char* g = reinterpret_cast<const char*>(src);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) cp_async_16(d + 16 * i, g + 16 * i);
  } else {
    for (int i = threadIdx.x; i < count; i += blockDim.x)
      cp_async_small<(int)sizeof(T)>(dst + i, src + i);
  }
}

// Device view of one line plan (passed by value in kernel parameters).
template <typename R>
struct LineDev {
  int n;        // logical length
  int nf;       // transform length of the core (n, or Bluestein m)
  int ld;       // shared-memory stride of one line (padded, >= sp(nf - 1) + 1)
  int blue;     // 1: Bluestein
  int nst;      // number of radix stages of the core
  int lg2;      // log2(nf) when the core runs the compile-time power-of-two
                // stages (kP2Min <= lg2 <= kP2Max), else 0
  int mixed;    // nf of a compile-time mixed-radix core (255 = 3.5.17), else 0
  int rad[kMaxStages];
  FastDiv dnbl[kMaxStages];  // stage s: division by nf / rad[s] (butterflies per line)
  FastDiv dms[kMaxStages];   // stage s: division by the butterfly span ms_s
  FastDiv dn, dnf;           // division by n, nf
  const cplx<R>* tw;     // nf entries, W_nf^k = exp(-2 pi i k / nf)
  const cplx<R>* chirp;  // n entries, exp(-i pi j^2 / n)      (Bluestein)
  const cplx<R>* bhat;   // nf entries, filter spectrum / nf, digit-reversed (Bluestein)
  const int* pos;        // n entries, frequency -> slot after the forward core (direct)
};

// ---------------------------------------------------------------------------
// radix-r DFTs on registers (forward sign -; inverse = conj o forward o conj)
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void dft2(cplx<R>* v) {
  cplx<R> a = v[0], b = v[1];
  v[0] = cadd<R>(a, b);
  v[1] = csub<R>(a, b);
}

template <typename R>
__device__ __forceinline__ void dft3(cplx<R>* v) {
  const R h = R(0.86602540378443864676372317075294);  // sqrt(3)/2
  cplx<R> s = cadd<R>(v[1], v[2]);
  cplx<R> d = csub<R>(v[1], v[2]);
  cplx<R> t1 = mkc<R>(v[0].x - R(0.5) * s.x, v[0].y - R(0.5) * s.y);
  cplx<R> t2 = mkc<R>(h * d.x, h * d.y);
  v[0] = cadd<R>(v[0], s);
  v[1] = cadd<R>(t1, cmul_mi<R>(t2));
  v[2] = cadd<R>(t1, cmul_pi<R>(t2));
}

template <typename R>
__device__ __forceinline__ void dft4(cplx<R>* v) {
  cplx<R> a = cadd<R>(v[0], v[2]), b = csub<R>(v[0], v[2]);
  cplx<R> c = cadd<R>(v[1], v[3]), d = csub<R>(v[1], v[3]);
  v[0] = cadd<R>(a, c);
  v[2] = csub<R>(a, c);
  v[1] = cadd<R>(b, cmul_mi<R>(d));
  v[3] = cadd<R>(b, cmul_pi<R>(d));
}

template <typename R>
__device__ __forceinline__ void dft5(cplx<R>* v) {
  const R c1 = R(0.30901699437494742410229341718282);   // cos(2pi/5)
  const R c2 = R(-0.80901699437494742410229341718282);  // cos(4pi/5)
  const R s1 = R(0.95105651629515357211643933337938);   // sin(2pi/5)
  const R s2 = R(0.58778525229247312916870595463907);   // sin(4pi/5)
  cplx<R> t1 = cadd<R>(v[1], v[4]), t3 = csub<R>(v[1], v[4]);
  cplx<R> t2 = cadd<R>(v[2], v[3]), t4 = csub<R>(v[2], v[3]);
  cplx<R> x0 = v[0];
  cplx<R> a1 = mkc<R>(x0.x + c1 * t1.x + c2 * t2.x, x0.y + c1 * t1.y + c2 * t2.y);
  cplx<R> a2 = mkc<R>(x0.x + c2 * t1.x + c1 * t2.x, x0.y + c2 * t1.y + c1 * t2.y);
  cplx<R> b1 = mkc<R>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  cplx<R> b2 = mkc<R>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  v[0] = mkc<R>(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
  v[1] = cadd<R>(a1, cmul_mi<R>(b1));
  v[4] = cadd<R>(a1, cmul_pi<R>(b1));
  v[2] = cadd<R>(a2, cmul_mi<R>(b2));
  v[3] = cadd<R>(a2, cmul_pi<R>(b2));
}

template <typename R>
__device__ __forceinline__ void dft8(cplx<R>* v) {
  const R r = R(0.70710678118654752440084436210485);
  cplx<R> e[4] = {v[0], v[2], v[4], v[6]};
  cplx<R> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<R>(e);
  dft4<R>(o);
  // o[k] *= W8^k
  o[1] = mkc<R>(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x));
  o[2] = cmul_mi<R>(o[2]);
  o[3] = mkc<R>(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd<R>(e[k], o[k]);
    v[k + 4] = csub<R>(e[k], o[k]);
  }
}

// ENDS: only x[0..3] and x[12..15] are nonzero (the band of a pruned
// 32-point line), so the first DFT4 of each b sees (x_b, 0, 0, x_{b+12}).
// OUT_ENDS: only X[0..3] and X[12..15] are wanted (outputs 0 and 3 of each
// last DFT4); X[4..11] are left unspecified.
template <typename R, bool ENDS = false, bool OUT_ENDS = false>
__device__ __forceinline__ void dft16(cplx<R>* v) {
  // x[b + 4a]: u_b = DFT4_a, twiddle W16^(b k1), then DFT4 over b.
  const R c1 = R(0.92387953251128675612818318939679);  // cos(pi/8)
  const R s1 = R(0.38268343236508977172845998403040);  // sin(pi/8)
  const R r = R(0.70710678118654752440084436210485);
  cplx<R> u[4][4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    if constexpr (ENDS) {
      const cplx<R> x0 = v[b], x3 = v[b + 12];
      u[b][0] = cadd<R>(x0, x3);
      u[b][1] = cadd<R>(x0, cmul_pi<R>(x3));
      u[b][2] = csub<R>(x0, x3);
      u[b][3] = csub<R>(x0, cmul_pi<R>(x3));
    } else {
      cplx<R> t[4] = {v[b], v[b + 4], v[b + 8], v[b + 12]};
      dft4<R>(t);
#pragma unroll
      for (int k = 0; k < 4; ++k) u[b][k] = t[k];
    }
  }
  // W16^1 = (c1,-s1), W16^2 = (r,-r), W16^3 = (s1,-c1), W16^4 = -i,
  // W16^6 = (-r,-r), W16^9 = (-c1,+s1)
  u[1][1] = cmul<R>(u[1][1], mkc<R>(c1, -s1));
  u[1][2] = cmul<R>(u[1][2], mkc<R>(r, -r));
  u[1][3] = cmul<R>(u[1][3], mkc<R>(s1, -c1));
  u[2][1] = cmul<R>(u[2][1], mkc<R>(r, -r));
  u[2][2] = cmul_mi<R>(u[2][2]);
  u[2][3] = cmul<R>(u[2][3], mkc<R>(-r, -r));
  u[3][1] = cmul<R>(u[3][1], mkc<R>(s1, -c1));
  u[3][2] = cmul<R>(u[3][2], mkc<R>(-r, -r));
  u[3][3] = cmul<R>(u[3][3], mkc<R>(-c1, s1));
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    if constexpr (OUT_ENDS) {
      const cplx<R> a = cadd<R>(u[0][k1], u[2][k1]), b = csub<R>(u[0][k1], u[2][k1]);
      const cplx<R> c = cadd<R>(u[1][k1], u[3][k1]), d = csub<R>(u[1][k1], u[3][k1]);
      v[k1] = cadd<R>(a, c);
      v[k1 + 12] = cadd<R>(b, cmul_pi<R>(d));
    } else {
      cplx<R> t[4] = {u[0][k1], u[1][k1], u[2][k1], u[3][k1]};
      dft4<R>(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
    }
  }
}

// 32 = 2 x 16: X[k] = E[k] + W32^k O[k], X[k+16] = E[k] - W32^k O[k] with E, O
// the 16-point DFTs of the even and odd samples (natural order in and out).
// ZIN: inputs 8..23 are zero (inverse span-1 stage of a band-pruned line);
// HALF: only outputs 0..7 and 24..31 are wanted (forward span-1 stage), the
// others are left unspecified.
template <typename R, bool ZIN = false, bool HALF = false>
__device__ __forceinline__ void dft32(cplx<R>* v) {
  const R c16 = R(0.98078528040323044912618223613424);   // cos(pi/16)
  const R s16 = R(0.19509032201612826784828486847702);   // sin(pi/16)
  const R c316 = R(0.83146961230254523707878837761791);  // cos(3pi/16)
  const R s316 = R(0.55557023301960222474283081394853);  // sin(3pi/16)
  const R c8 = R(0.92387953251128675612818318939679);    // cos(pi/8)
  const R s8 = R(0.38268343236508977172845998403040);    // sin(pi/8)
  const R r = R(0.70710678118654752440084436210485);
  cplx<R> e[16], o[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    e[k] = v[2 * k];
    o[k] = v[2 * k + 1];
  }
  dft16<R, ZIN>(e);
  dft16<R, ZIN>(o);
  // o[k] *= W32^k = (cos(pi k/16), -sin(pi k/16))
  o[1] = cmul<R>(o[1], mkc<R>(c16, -s16));
  o[2] = cmul<R>(o[2], mkc<R>(c8, -s8));
  o[3] = cmul<R>(o[3], mkc<R>(c316, -s316));
  o[4] = cmul<R>(o[4], mkc<R>(r, -r));
  o[5] = cmul<R>(o[5], mkc<R>(s316, -c316));
  o[6] = cmul<R>(o[6], mkc<R>(s8, -c8));
  o[7] = cmul<R>(o[7], mkc<R>(s16, -c16));
  o[8] = cmul_mi<R>(o[8]);
  o[9] = cmul<R>(o[9], mkc<R>(-s16, -c16));
  o[10] = cmul<R>(o[10], mkc<R>(-s8, -c8));
  o[11] = cmul<R>(o[11], mkc<R>(-s316, -c316));
  o[12] = cmul<R>(o[12], mkc<R>(-r, -r));
  o[13] = cmul<R>(o[13], mkc<R>(-c316, -s316));
  o[14] = cmul<R>(o[14], mkc<R>(-c8, -s8));
  o[15] = cmul<R>(o[15], mkc<R>(-c16, -s16));
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    if (!HALF || k < 8) v[k] = cadd<R>(e[k], o[k]);
    if (!HALF || k >= 8) v[k + 16] = csub<R>(e[k], o[k]);
  }
}

// cos(2 pi m / r) and sin(2 pi m / r), m = 1 .. (r-1)/2, of the odd prime
// radices (evaluated in 50-digit decimal arithmetic from Machin's pi and
// the Taylor series), so the DFT_r constants are immediates, not table loads.
template <int RAD>
__host__ __device__ constexpr double odd_root_cos(int m) {
  if constexpr (RAD == 7) {
    constexpr double t[3] = {6.234898018587335305250e-1, -2.225209339563144042889e-1, -9.009688679024191262361e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 11) {
    constexpr double t[5] = {8.412535328311811688618e-1, 4.154150130018864255293e-1, -1.423148382732851404438e-1, -6.548607339452850640569e-1, -9.594929736144973898904e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 13) {
    constexpr double t[6] = {8.854560256532098959004e-1, 5.680647467311558025118e-1, 1.205366802553230533491e-1, -3.546048870425356259696e-1, -7.485107481711010986346e-1, -9.709418174260520271570e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 17) {
    constexpr double t[8] = {9.324722294043558045731e-1, 7.390089172206591159245e-1, 4.457383557765382673965e-1, 9.226835946330199523965e-2, -2.736629900720828635391e-1, -6.026346363792563891786e-1, -8.502171357296141521341e-1, -9.829730996839017782819e-1};
    return t[m - 1];
  }
  return 0.0;
}
template <int RAD>
__host__ __device__ constexpr double odd_root_sin(int m) {
  if constexpr (RAD == 7) {
    constexpr double t[3] = {7.818314824680298087084e-1, 9.749279121818236070181e-1, 4.338837391175581204758e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 11) {
    constexpr double t[5] = {5.406408174555975821076e-1, 9.096319953545183714117e-1, 9.898214418809327323761e-1, 7.557495743542582837740e-1, 2.817325568414296977114e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 13) {
    constexpr double t[6] = {4.647231720437685456560e-1, 8.229838658936563945796e-1, 9.927088740980539928008e-1, 9.350162426854148234398e-1, 6.631226582407952023768e-1, 2.393156642875577671488e-1};
    return t[m - 1];
  }
  if constexpr (RAD == 17) {
    constexpr double t[8] = {3.612416661871529487447e-1, 6.736956436465572117127e-1, 8.951632913550623220670e-1, 9.957341762950345218712e-1, 9.618256431728190704088e-1, 7.980172272802395033328e-1, 5.264321628773558002446e-1, 1.837495178165703315744e-1};
    return t[m - 1];
  }
  return 0.0;
}

// Odd prime radix, symmetric-pair form, in place: v[j] <- v[j] + v[r-j] and
// v[r-j] <- v[j] - v[r-j] for j <= (r-1)/2, then the outputs pair up as
// y_k = a_k - i b_k, y_{r-k} = a_k + i b_k with a_k = x0 + sum_j cos(2pi jk/r) s_j,
// b_k = sum_j sin(2pi jk/r) d_j, with the constants of odd_root_cos/sin.
// Only the r input registers and two accumulators stay live.
template <typename R, int RAD>
__device__ __forceinline__ void dft_odd(cplx<R>* v, const cplx<R>* __restrict__ tw, int nf) {
  constexpr int H = (RAD - 1) / 2;
  (void)tw;
  (void)nf;
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    const cplx<R> a = v[j], b = v[RAD - j];
    v[j] = cadd<R>(a, b);
    v[RAD - j] = csub<R>(a, b);
  }
  const cplx<R> x0 = v[0];
  cplx<R> y0 = x0;
#pragma unroll
  for (int j = 1; j <= H; ++j) y0 = cadd<R>(y0, v[j]);
  // outputs are written back in place after all sums that need the inputs:
  // compute pairs into a small rolling buffer of H values each
  cplx<R> ak[H], bk[H];
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    cplx<R> a = x0;
    cplx<R> b = mkc<R>(R(0), R(0));
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      // m = jk mod r folded into 1..H: cos is even, sin odd about r/2
      const int m = (j * k) % RAD;
      const R c = (R)odd_root_cos<RAD>(m <= H ? m : RAD - m);
      const R sn = m <= H ? (R)odd_root_sin<RAD>(m) : -(R)odd_root_sin<RAD>(RAD - m);
      a.x += c * v[j].x;
      a.y += c * v[j].y;
      b.x += sn * v[RAD - j].x;
      b.y += sn * v[RAD - j].y;
    }
    ak[k - 1] = a;
    bk[k - 1] = b;
  }
  v[0] = y0;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    v[k] = cadd<R>(ak[k - 1], cmul_mi<R>(bk[k - 1]));
    v[RAD - k] = cadd<R>(ak[k - 1], cmul_pi<R>(bk[k - 1]));
  }
}

template <typename R, int RAD>
__device__ __forceinline__ void dft_fwd(cplx<R>* v, const cplx<R>* __restrict__ tw, int nf) {
  if constexpr (RAD == 2) dft2<R>(v);
  else if constexpr (RAD == 3) dft3<R>(v);
  else if constexpr (RAD == 4) dft4<R>(v);
  else if constexpr (RAD == 5) dft5<R>(v);
  else if constexpr (RAD == 8) dft8<R>(v);
  else if constexpr (RAD == 16) dft16<R>(v);
  else if constexpr (RAD == 32) dft32<R>(v);
  else dft_odd<R, RAD>(v, tw, nf);
}

// ---------------------------------------------------------------------------
// radix stages over a batch of lines in shared memory
// ---------------------------------------------------------------------------
// Forward DIF stage on sub-arrays of length ns: butterfly (g, j1) reads
// slots g*ns + j1 + q*ms, applies DFT_r, multiplies output p by W_ns^(j1 p).
template <typename R, int RAD, bool INV>
__device__ __forceinline__ void stage_run(cplx<R>* __restrict__ buf, int ld, int nlines, int nf,
                                          int ns, const cplx<R>* __restrict__ tw, int tid,
                                          int nthr, FastDiv dnbl, FastDiv dms) {
  const int ms = ns / RAD;
  const int nbl = nf / RAD;
  const int tws = nf / ns;
  if constexpr (RAD > 8 && RAD != 16) {
    // odd radices above 8: one (line, butterfly) pair per step, nothing kept
    // across lines (their slot offsets would not fit the register budget).
    // A span-1 stage (ms = 1, the last DIF stage) has only unit twiddles.
    const int total = nlines * nbl;
    const bool tw1 = ms == 1;
    for (int b = tid; b < total; b += nthr) {
      const int line = fdiv(b, dnbl);
      const int bb = b - line * nbl;
      const int g = tw1 ? bb : fdiv(bb, dms);
      const int j1 = bb - g * ms;
      cplx<R>* lp = buf + line * ld;
      const int base = g * ns + j1;
      cplx<R> v[RAD];
      if constexpr (!INV) {
#pragma unroll
        for (int q = 0; q < RAD; ++q) v[q] = lp[sp(base + q * ms)];
        dft_fwd<R, RAD>(v, tw, nf);
        lp[sp(base)] = v[0];
        if (tw1) {
#pragma unroll
          for (int q = 1; q < RAD; ++q) lp[sp(base + q)] = v[q];
        } else {
#pragma unroll
          for (int q = 1; q < RAD; ++q) lp[sp(base + q * ms)] = cmul<R>(v[q], tw[j1 * q * tws]);
        }
      } else {
        v[0] = cconj<R>(lp[sp(base)]);
        if (tw1) {
#pragma unroll
          for (int q = 1; q < RAD; ++q) v[q] = cconj<R>(lp[sp(base + q)]);
        } else {
#pragma unroll
          for (int q = 1; q < RAD; ++q)
            v[q] = cconj<R>(cmulc<R>(lp[sp(base + q * ms)], tw[j1 * q * tws]));
        }
        dft_fwd<R, RAD>(v, tw, nf);
#pragma unroll
        for (int q = 0; q < RAD; ++q) lp[sp(base + q * ms)] = cconj<R>(v[q]);
      }
    }
    return;
  }
  // Butterfly-stationary: a thread keeps one butterfly position (its slots
  // and twiddles) and runs it over a strided subset of the lines, so the index
  // arithmetic and twiddle loads are paid once per stage, not once per line.
  int bb0 = tid, bstep = nthr, l0 = 0, lstep = 1;
  if (nbl < nthr) {
    lstep = fdiv(nthr, dnbl);  // groups of nbl threads
    l0 = fdiv(tid, dnbl);
    bb0 = tid - l0 * nbl;
    bstep = nbl;
    if (l0 >= lstep) return;
  }
  constexpr bool kCacheTw = RAD <= 8;  // registers: larger radices reload per line
  for (int bb = bb0; bb < nbl; bb += bstep) {
    const int g = fdiv(bb, dms);
    const int j1 = bb - g * ms;
    const int base = g * ns + j1;
    cplx<R> w[RAD];
    if constexpr (kCacheTw) {
#pragma unroll
      for (int q = 1; q < RAD; ++q) w[q] = tw[j1 * q * tws];
    }
    for (int line = l0; line < nlines; line += lstep) {
      cplx<R>* lp = buf + line * ld;
      cplx<R> v[RAD];
      if constexpr (!INV) {
#pragma unroll
        for (int q = 0; q < RAD; ++q) v[q] = lp[sp(base + q * ms)];
        dft_fwd<R, RAD>(v, tw, nf);
        lp[sp(base)] = v[0];
#pragma unroll
        for (int q = 1; q < RAD; ++q)
          lp[sp(base + q * ms)] = cmul<R>(v[q], kCacheTw ? w[q] : tw[j1 * q * tws]);
      } else {
        v[0] = cconj<R>(lp[sp(base)]);
#pragma unroll
        for (int q = 1; q < RAD; ++q)
          v[q] = cconj<R>(cmulc<R>(lp[sp(base + q * ms)], kCacheTw ? w[q] : tw[j1 * q * tws]));
        dft_fwd<R, RAD>(v, tw, nf);
#pragma unroll
        for (int q = 0; q < RAD; ++q) lp[sp(base + q * ms)] = cconj<R>(v[q]);
      }
    }
  }
}

// Radix dispatch, inlined into every FFT kernel (no call, so no call-frame
// registers or stack).  Lengths with a prime factor above 17 go through
// Bluestein (build_line_plan), so these are all the radices a plan can hold.
template <typename R, bool INV>
__device__ __forceinline__ void stage_dispatch(cplx<R>* buf, int ld, int nlines, int nf, int ns,
                                               int rad, const cplx<R>* tw, int tid, int nthr,
                                               FastDiv dnbl, FastDiv dms) {
  switch (rad) {
    case 2: stage_run<R, 2, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 3: stage_run<R, 3, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 4: stage_run<R, 4, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 5: stage_run<R, 5, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 7: stage_run<R, 7, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 8: stage_run<R, 8, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 11: stage_run<R, 11, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 13: stage_run<R, 13, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 16: stage_run<R, 16, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    case 17: stage_run<R, 17, INV>(buf, ld, nlines, nf, ns, tw, tid, nthr, dnbl, dms); break;
    default: break;  // plans only contain the radices of factor_radices
  }
}

// ---------------------------------------------------------------------------
// Power-of-two cores with a compile-time stage sequence.  The radices are
// those of factor_radices (2^P in ceil(P/4) stages, exponents as even as
// possible, the larger ones first: 512 = 8.8.8, 1024 = 16.8.8, 256 = 16.16;
// FP32 512 = 16.32, see p2_k_for),
// and the slots and twiddles are the run-time path's, so the digit-reversed
// positions (LineDev::pos) and the arithmetic are unchanged.  What changes is
// the index work: butterfly coordinates are shifts and masks, and the r slots
// of a butterfly sit at compile-time offsets from its first slot, because for
// power-of-two spans sp(g*ns + j1 + q*ms) = sp(g*ns + j1) + sp(q*ms) (adding
// q*ms never carries across a 32-slot boundary of the padding).
// ---------------------------------------------------------------------------
// FP32 cores of 2^kP2TwoStageLg points run as two stages (K = 2 below); the
// host plans them with factor_radices(..., two_stage_len = 1 << kP2TwoStageLg)
// so LineDev::pos and Bluestein's bhat follow the same digit order.  FP64
// keeps the default stages, whose butterflies fit its registers.
constexpr int kP2TwoStageLg = 9;
template <typename R>
__host__ __device__ constexpr int p2_k_for(int P) {
  return (sizeof(R) == 4 && P == kP2TwoStageLg) ? 2 : 0;
}
template <typename R>
constexpr int p2_two_stage_len() {
  return sizeof(R) == 4 ? (1 << kP2TwoStageLg) : 0;
}

// Stage decomposition of a 2^P core, stage s taking e(s) bits of the index.
// K = 0: ceil(P/4) stages of radix <= 16, larger radices first (the run-time
// path's order, so LineDev::pos holds).  K = 2: two stages with the larger
// radix last (512 = 16 . 32): the last DIF stage has span 1, so the radix-32
// butterflies need no twiddles and carry the band pruning, and a line takes
// three shared-memory passes (inverse, fused middle, forward) instead of five.
__host__ __device__ constexpr int p2_nst(int P, int K = 0) { return K ? K : (P + 3) / 4; }
__host__ __device__ constexpr int p2_e(int P, int s, int K = 0) {
  return K ? P / K + (s >= K - P % K ? 1 : 0)
           : P / p2_nst(P) + (s < P % p2_nst(P) ? 1 : 0);
}
__host__ __device__ constexpr int p2_ebefore(int P, int s, int K = 0) {
  int t = 0;
  for (int i = 0; i < s; ++i) t += p2_e(P, i, K);
  return t;
}
// slot of frequency k after the forward DIF of length 2^P (digit reversal)
template <int P, int K = 0>
__device__ __forceinline__ int p2_pos(int k) {
  int pos = 0;
#pragma unroll
  for (int s = 0; s < p2_nst(P, K); ++s) {
    const int e = p2_e(P, s, K), eb = p2_ebefore(P, s, K);
    pos |= ((k >> eb) & ((1 << e) - 1)) << (P - eb - e);
  }
  return pos;
}

// Stage S of the in-place DIF (forward) or its inverse, on nlines lines.
// A thread keeps one butterfly (its slots and twiddles) for all its lines;
// requires blockDim.x to be a multiple of the butterflies per line (every
// launch uses 256 threads; the largest count is 128).  Stages of span 1 (the
// last DIF / first DIT stage) have only the unit twiddle and skip the multiply.
// PRUNE (span-1 stage of a line whose spectrum is zero for N/4 <= k <= 3N/4):
// digits q in [RAD/4, 3 RAD/4) of such a butterfly are those frequencies, so
// the inverse reads them as zeros and the forward does not store them.
template <int RAD>
__host__ __device__ constexpr bool p2_pruned_digit(int q) {
  return q >= RAD / 4 && q < 3 * RAD / 4;
}

template <typename R, int P, int S, bool INV, bool PRUNE = false, int K = 0>
__device__ __forceinline__ void p2_stage(cplx<R>* __restrict__ buf, int ld, int nlines,
                                         const cplx<R>* __restrict__ tw) {
  constexpr int E = p2_e(P, S, K), EB = p2_ebefore(P, S, K);
  constexpr int RAD = 1 << E;
  constexpr int LNS = P - EB, LMS = LNS - E, LNBL = P - E;
  constexpr int NS = 1 << LNS, MS = 1 << LMS, NBL = 1 << LNBL;
  constexpr bool TW = MS > 1;
  static_assert(NBL <= 256, "butterflies per line exceed the CTA");
  static_assert(!PRUNE || (!TW && RAD >= 4), "pruning applies to span-1 stages");
  const int tid = threadIdx.x;
  const int lstep = blockDim.x >> LNBL;
  const int l0 = tid >> LNBL;
  const int bb = tid & (NBL - 1);
  const int g = bb >> LMS, j1 = bb & (MS - 1);
  const int sbase = sp(g * NS + j1);
  cplx<R> w[RAD];
  if constexpr (TW) {
#pragma unroll
    for (int q = 1; q < RAD; ++q) w[q] = tw[(j1 * q) << EB];
  }
  for (int line = l0; line < nlines; line += lstep) {
    cplx<R>* lp = buf + line * ld + sbase;
    cplx<R> v[RAD];
    if constexpr (!INV) {
#pragma unroll
      for (int q = 0; q < RAD; ++q) v[q] = lp[sp(q * MS)];
      if constexpr (PRUNE && RAD == 32) dft32<R, false, true>(v);
      else dft_fwd<R, RAD>(v, tw, 1 << P);
      lp[0] = v[0];
#pragma unroll
      for (int q = 1; q < RAD; ++q) {
        if (PRUNE && p2_pruned_digit<RAD>(q)) continue;
        lp[sp(q * MS)] = TW ? cmul<R>(v[q], w[q]) : v[q];
      }
    } else {
      v[0] = cconj<R>(lp[0]);
#pragma unroll
      for (int q = 1; q < RAD; ++q) {
        if (PRUNE && p2_pruned_digit<RAD>(q)) v[q] = mkc<R>(R(0), R(0));
        else v[q] = TW ? cconj<R>(cmulc<R>(lp[sp(q * MS)], w[q])) : cconj<R>(lp[sp(q * MS)]);
      }
      if constexpr (PRUNE && RAD == 32) dft32<R, true, false>(v);
      else dft_fwd<R, RAD>(v, tw, 1 << P);
#pragma unroll
      for (int q = 0; q < RAD; ++q) lp[sp(q * MS)] = cconj<R>(v[q]);
    }
  }
}

// PRUNE: the span-1 stage (S = NST-1) skips the digits of N/4 <= k < 3N/4
// (inverse: zero inputs, forward: unused outputs); see p2_stage.
template <typename R, int P, bool INV, bool PRUNE = false, int K = 0>
__device__ __forceinline__ void p2_run(cplx<R>* buf, int ld, int nlines, const cplx<R>* tw) {
  constexpr int NST = p2_nst(P, K);
  static_assert(NST >= 2 && NST <= 3, "power-of-two cores 2^5 .. 2^12");
  if constexpr (!INV) {
    p2_stage<R, P, 0, false, false, K>(buf, ld, nlines, tw);
    __syncthreads();
    if constexpr (NST > 2) { p2_stage<R, P, 1, false, false, K>(buf, ld, nlines, tw); __syncthreads(); }
    p2_stage<R, P, NST - 1, false, PRUNE, K>(buf, ld, nlines, tw);
    __syncthreads();
  } else {
    p2_stage<R, P, NST - 1, true, PRUNE, K>(buf, ld, nlines, tw);
    __syncthreads();
    if constexpr (NST > 2) { p2_stage<R, P, 1, true, false, K>(buf, ld, nlines, tw); __syncthreads(); }
    p2_stage<R, P, 0, true, false, K>(buf, ld, nlines, tw);
    __syncthreads();
  }
}

// prune: a direct line whose spectrum is zero (inverse) or not read (forward)
// for N/4 <= k < 3N/4; ignored for Bluestein lines
template <typename R, int P>
__device__ __forceinline__ void line_core_p2(cplx<R>* buf, int ld, int nlines, const LineDev<R>& L,
                                             bool inverse, bool prune = false) {
  constexpr int K = p2_k_for<R>(P);
  if (prune && !L.blue) {
    if (inverse) p2_run<R, P, true, true, K>(buf, ld, nlines, L.tw);
    else p2_run<R, P, false, true, K>(buf, ld, nlines, L.tw);
    return;
  }
  if (L.blue || !inverse) p2_run<R, P, false, false, K>(buf, ld, nlines, L.tw);
  if (L.blue) {
    const int tot = nlines << P;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int line = e >> P, j = e & ((1 << P) - 1);
      cplx<R>* p = buf + line * ld + sp(j);
      *p = cmul<R>(*p, L.bhat[j]);
    }
    __syncthreads();
  }
  if (L.blue || inverse) p2_run<R, P, true, false, K>(buf, ld, nlines, L.tw);
}

// ---------------------------------------------------------------------------
// Compile-time mixed-radix core for a direct line of length prod(RADS...) with
// the radices in the order of factor_radices (so LineDev::pos stays valid):
// 255 = 3.5.17, the solve-grid lines of the 255^3 image.  Butterfly
// coordinates are divisions by compile-time constants; a thread computes its
// butterfly's slots (and twiddles, for spans above 1) once per stage.
// Requires blockDim.x >= N / RAD for every stage (at most 85 here).
// ---------------------------------------------------------------------------
template <typename R, int N, int RAD, int NS, bool INV>
__device__ __forceinline__ void mixed_stage(cplx<R>* __restrict__ buf, int ld, int nlines,
                                            const cplx<R>* __restrict__ tw) {
  constexpr int MS = NS / RAD, NBL = N / RAD, TWS = N / NS;
  constexpr bool TW = MS > 1;
  const int tid = threadIdx.x;
  const int lstep = (int)blockDim.x / NBL;
  const int l0 = tid / NBL;
  if (l0 >= lstep) return;
  const int bb = tid - l0 * NBL;
  const int g = bb / MS, j1 = bb - g * MS;
  const int base = g * NS + j1;
  int slot[RAD];
#pragma unroll
  for (int q = 0; q < RAD; ++q) slot[q] = sp(base + q * MS);
  cplx<R> w[RAD];
  if constexpr (TW) {
#pragma unroll
    for (int q = 1; q < RAD; ++q) w[q] = tw[j1 * q * TWS];
  }
  for (int line = l0; line < nlines; line += lstep) {
    cplx<R>* lp = buf + line * ld;
    cplx<R> v[RAD];
    if constexpr (!INV) {
#pragma unroll
      for (int q = 0; q < RAD; ++q) v[q] = lp[slot[q]];
      dft_fwd<R, RAD>(v, tw, N);
      lp[slot[0]] = v[0];
#pragma unroll
      for (int q = 1; q < RAD; ++q) lp[slot[q]] = TW ? cmul<R>(v[q], w[q]) : v[q];
    } else {
      v[0] = cconj<R>(lp[slot[0]]);
#pragma unroll
      for (int q = 1; q < RAD; ++q)
        v[q] = TW ? cconj<R>(cmulc<R>(lp[slot[q]], w[q])) : cconj<R>(lp[slot[q]]);
      dft_fwd<R, RAD>(v, tw, N);
#pragma unroll
      for (int q = 0; q < RAD; ++q) lp[slot[q]] = cconj<R>(v[q]);
    }
  }
}

// 255 = 3.5.17: spans 255 / 85 / 17 with butterfly spans 85 / 17 / 1
template <typename R>
__device__ __forceinline__ void line_core_255(cplx<R>* buf, int ld, int nlines,
                                              const cplx<R>* tw, bool inverse) {
  if (!inverse) {
    mixed_stage<R, 255, 3, 255, false>(buf, ld, nlines, tw);
    __syncthreads();
    mixed_stage<R, 255, 5, 85, false>(buf, ld, nlines, tw);
    __syncthreads();
    mixed_stage<R, 255, 17, 17, false>(buf, ld, nlines, tw);
    __syncthreads();
  } else {
    mixed_stage<R, 255, 17, 17, true>(buf, ld, nlines, tw);
    __syncthreads();
    mixed_stage<R, 255, 5, 85, true>(buf, ld, nlines, tw);
    __syncthreads();
    mixed_stage<R, 255, 3, 255, true>(buf, ld, nlines, tw);
    __syncthreads();
  }
}

// A line of length nf = 2^P (direct, compile-time core) whose nonzero or used
// frequencies satisfy |q| <= hq can skip the digits of N/4 <= k < 3N/4 in its
// span-1 stage: k = q <= hq < N/4 and k = N - q >= N - hq > 3N/4.
template <typename R>
__device__ __forceinline__ bool line_prunable(const LineDev<R>& L, int hq) {
  return L.lg2 > 0 && !L.blue && 4 * hq < L.nf;
}

// Core transform of nlines lines (length L.nf each, stride ld) in place.
//   direct, forward : DIF            (natural -> digit-reversed)
//   direct, inverse : DIT^-1         (digit-reversed -> natural), unnormalised
//   Bluestein (either direction, conjugations at put/get): DIF, * bhat, DIT^-1
// Ends with __syncthreads().
// prune (power-of-two direct lines only, see line_prunable): the caller's
// spectrum is zero / unused for N/4 <= k < 3N/4.
template <typename R>
__device__ void line_core(cplx<R>* buf, int ld, int nlines, const LineDev<R>& L, bool inverse,
                          bool prune = false) {
  static_assert(kP2Min == 5 && kP2Max == 10, "dispatch below lists 2^5 .. 2^10");
  switch (L.lg2) {
    case 5: line_core_p2<R, 5>(buf, ld, nlines, L, inverse, prune); return;
    case 6: line_core_p2<R, 6>(buf, ld, nlines, L, inverse, prune); return;
    case 7: line_core_p2<R, 7>(buf, ld, nlines, L, inverse, prune); return;
    case 8: line_core_p2<R, 8>(buf, ld, nlines, L, inverse, prune); return;
    case 9: line_core_p2<R, 9>(buf, ld, nlines, L, inverse, prune); return;
    case 10: line_core_p2<R, 10>(buf, ld, nlines, L, inverse, prune); return;
    default: break;
  }
  if (L.mixed == 255) {
    line_core_255<R>(buf, ld, nlines, L.tw, inverse);
    return;
  }
  const int tid = threadIdx.x, nthr = blockDim.x;
  const bool do_fwd = L.blue || !inverse;
  const bool do_inv = L.blue || inverse;
  if (do_fwd) {
    int ns = L.nf;
    for (int s = 0; s < L.nst; ++s) {
      stage_dispatch<R, false>(buf, ld, nlines, L.nf, ns, L.rad[s], L.tw, tid, nthr, L.dnbl[s],
                               L.dms[s]);
      ns /= L.rad[s];
      __syncthreads();
    }
  }
  if (L.blue) {
    const int tot = nlines * L.nf;
    for (int e = tid; e < tot; e += nthr) {
      const int line = fdiv(e, L.dnf), j = e - line * L.nf;
      cplx<R>* p = buf + line * ld + sp(j);
      *p = cmul<R>(*p, L.bhat[j]);
    }
    __syncthreads();
  }
  if (do_inv) {
    // stage sizes: ns_s = nf / (r_0 ... r_{s-1}); run s = nst-1 .. 0
    int ns = 1;
    for (int s = L.nst - 1; s >= 0; --s) {
      ns *= L.rad[s];
      stage_dispatch<R, true>(buf, ld, nlines, L.nf, ns, L.rad[s], L.tw, tid, nthr, L.dnbl[s],
                              L.dms[s]);
      __syncthreads();
    }
  }
}

// --- value placement in frequency / space order -----------------------------
// forward input x_j (natural, j < n)
template <typename R>
__device__ __forceinline__ void put_fwd(cplx<R>* line, const LineDev<R>& L, int j, cplx<R> v) {
  line[sp(j)] = L.blue ? cmul<R>(v, L.chirp[j]) : v;
}
// digit-reversed slot of frequency k in a direct line: shifts and masks when
// the line runs the compile-time power-of-two stages (the same positions as
// the plan's table), the table otherwise
template <typename R>
__device__ __forceinline__ int line_pos(const LineDev<R>& L, int k) {
  switch (L.lg2) {
    case 5: return p2_pos<5, p2_k_for<R>(5)>(k);
    case 6: return p2_pos<6, p2_k_for<R>(6)>(k);
    case 7: return p2_pos<7, p2_k_for<R>(7)>(k);
    case 8: return p2_pos<8, p2_k_for<R>(8)>(k);
    case 9: return p2_pos<9, p2_k_for<R>(9)>(k);
    case 10: return p2_pos<10, p2_k_for<R>(10)>(k);
    default: return L.pos[k];
  }
}
// forward output X_k (k < n)
template <typename R>
__device__ __forceinline__ cplx<R> get_fwd(const cplx<R>* line, const LineDev<R>& L, int k) {
  return L.blue ? cmul<R>(line[sp(k)], L.chirp[k]) : line[sp(line_pos<R>(L, k))];
}
// inverse input X_k (k < n)
template <typename R>
__device__ __forceinline__ void put_inv(cplx<R>* line, const LineDev<R>& L, int k, cplx<R> v) {
  if (L.blue) line[sp(k)] = cmul<R>(cconj<R>(v), L.chirp[k]);
  else line[sp(line_pos<R>(L, k))] = v;
}
// inverse output x_j (j < n), unnormalised
template <typename R>
__device__ __forceinline__ cplx<R> get_inv(const cplx<R>* line, const LineDev<R>& L, int j) {
  return L.blue ? cconj<R>(cmul<R>(line[sp(j)], L.chirp[j])) : line[sp(j)];
}
// Asynchronous placement of a line input element straight into its slot
// (direct lines: a plain copy; Bluestein lines: the raw value, fixed up by
// blue_fixup after the copies complete).  slot_fwd / slot_inv give the slot
// of input element j of the forward / inverse core.
template <typename R>
__device__ __forceinline__ void cp_async_cplx(cplx<R>* smem, const cplx<R>* gmem) {
  if constexpr (sizeof(cplx<R>) == 16) cp_async_16(smem, gmem);
  else cp_async_small<8>(smem, gmem);
}
template <typename R>
__device__ __forceinline__ int slot_fwd(const LineDev<R>& L, int j) { return sp(j); }
template <typename R>
__device__ __forceinline__ int slot_inv(const LineDev<R>& L, int k) {
  return L.blue ? sp(k) : sp(line_pos<R>(L, k));
}
// Bluestein lines loaded raw into slots j < n: forward input x_j chirp_j,
// inverse input conj(X_k) chirp_k (what put_fwd / put_inv store).
template <typename R, bool INV>
__device__ __forceinline__ void blue_fixup(cplx<R>* buf, int ld, int nlines, const LineDev<R>& L) {
  if (!L.blue) return;
  const int tot = nlines * L.n;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int line = fdiv(e, L.dn), j = e - line * L.n;
    cplx<R>* p = buf + line * ld + sp(j);
    const cplx<R> v = *p;
    *p = INV ? cmul<R>(cconj<R>(v), L.chirp[j]) : cmul<R>(v, L.chirp[j]);
  }
}

// Bluestein lines need zeros in slots [n, nf) before the core.
template <typename R>
__device__ __forceinline__ void zero_tail(cplx<R>* buf, int ld, int nlines, const LineDev<R>& L) {
  if (!L.blue) return;
  const int lane = threadIdx.x & 31;
  for (int line = threadIdx.x >> 5; line < nlines; line += blockDim.x >> 5)
    for (int j = L.n + lane; j < L.nf; j += 32) buf[line * ld + sp(j)] = mkc<R>(R(0), R(0));
}

}  // namespace fhp
