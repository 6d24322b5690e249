// Line plans: radix factorisation, twiddles, Bluestein chirp/filter tables.
// All tables are computed in long double and rounded once to the working
// precision by the engine.
#include <cmath>
#include <complex>
#include <mutex>
#include <string>
#include <vector>

#include "fhp_engine.h"

namespace fhp {

namespace {
std::mutex g_err_mu;
std::string g_err;
const long double kPi = 3.141592653589793238462643383279502884L;

std::complex<long double> root(long long num, long long den) {
  // exp(-2 pi i num/den), num reduced mod den first
  long long r = num % den;
  if (r < 0) r += den;
  const long double a = 2.0L * kPi * (long double)r / (long double)den;
  return {std::cos(a), -std::sin(a)};
}
}  // namespace

void set_error(const std::string& msg) {
  std::lock_guard<std::mutex> g(g_err_mu);
  g_err = msg;
}
const char* last_error() {
  std::lock_guard<std::mutex> g(g_err_mu);
  return g_err.c_str();
}

int Profiler::kind_of(const std::string& name, double bytes) {
  for (size_t i = 0; i < kinds.size(); ++i)
    if (kinds[i].name == name) return (int)i;
  ProfEntry e;
  e.name = name;
  e.bytes = bytes;
  kinds.push_back(e);
  return (int)kinds.size() - 1;
}

static cudaEvent_t take_event(std::vector<cudaEvent_t>& pool) {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void Profiler::begin(int kind, cudaStream_t s) {
  Rec r{kind, take_event(pool), take_event(pool)};
  cudaEventRecord(r.a, s);
  recs.push_back(r);
}

void Profiler::end(cudaStream_t s) {
  if (!recs.empty()) cudaEventRecord(recs.back().b, s);
}

void Profiler::collect() {
  for (Rec& r : recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      kinds[r.kind].ms += ms;
      kinds[r.kind].launches += 1;
    }
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  recs.clear();
}

void Profiler::reset() {
  collect();
  for (ProfEntry& k : kinds) { k.launches = 0; k.ms = 0.0; }
}

Profiler::~Profiler() {
  for (Rec& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

bool factor_radices(int n, std::vector<int>& rad, int two_stage_len) {
  rad.clear();
  if (n < 1) return false;
  int m = n, p2 = 0;
  while (m % 2 == 0) { m /= 2; ++p2; }
  if (n == two_stage_len && m == 1 && p2 >= 2) {
    // two stages, the larger radix last (512 = 16 * 32): the device's
    // compile-time core for this length uses the same order
    rad.push_back(1 << (p2 / 2));
    rad.push_back(1 << (p2 - p2 / 2));
    return true;
  }
  // 2^p2 in the fewest stages of radix <= 16, exponents as even as possible
  // (512 = 8 * 8 * 8 rather than 16 * 16 * 2: no cheap radix-2 stage that costs
  // a full pass over shared memory)
  if (p2 > 0) {
    const int nst2 = (p2 + 3) / 4;
    for (int s = 0; s < nst2; ++s) {
      const int e = p2 / nst2 + (s < p2 % nst2 ? 1 : 0);
      rad.push_back(1 << e);
    }
  }
  for (int p : {3, 5, 7, 11, 13, 17})
    while (m % p == 0) { rad.push_back(p); m /= p; }
  return m == 1;
}

static bool smooth235(int m) {
  for (int p : {2, 3, 5}) while (m % p == 0) m /= p;
  return m == 1;
}

// slot of frequency k after the forward DIF with radices rad (length n)
static int dif_slot(int k, int n, const std::vector<int>& rad) {
  int P = 0, ns = n, kk = k;
  for (int r : rad) {
    const int ms = ns / r;
    P += (kk % r) * ms;
    kk /= r;
    ns = ms;
  }
  return P;
}

bool build_line_plan(int n, LinePlanHost& out, int two_stage_len) {
  out = LinePlanHost();
  out.n = n;
  std::vector<int> rad;
  if (n == 1) {
    out.nf = 1; out.blue = 0; out.nst = 0;
    out.pos = {0};
    out.tw = {1.0L};
    return true;
  }
  if (factor_radices(n, rad, two_stage_len)) {
    out.nf = n;
    out.blue = 0;
    out.rad = rad;
    out.nst = (int)rad.size();
    out.tw.resize(n);
    for (int k = 0; k < n; ++k) out.tw[k] = root(k, n);
    out.pos.resize(n);
    for (int k = 0; k < n; ++k) out.pos[k] = dif_slot(k, n, rad);
    return true;
  }
  // Bluestein: smallest 2^a 3^b 5^c >= 2n-1
  int m = 2 * n - 1;
  while (!smooth235(m)) ++m;
  if (!factor_radices(m, rad, two_stage_len)) return false;
  out.nf = m;
  out.blue = 1;
  out.rad = rad;
  out.nst = (int)rad.size();
  out.tw.resize(m);
  for (int k = 0; k < m; ++k) out.tw[k] = root(k, m);
  // chirp_j = exp(-i pi j^2 / n) = root(j^2 mod 2n, 2n)
  out.chirp.resize(n);
  for (int j = 0; j < n; ++j) {
    const long long t = ((long long)j * j) % (2LL * n);
    out.chirp[j] = root(t, 2LL * n);
  }
  // filter b_j = conj(chirp_j) for |j| < n (cyclic in m)
  std::vector<std::complex<long double>> b(m, 0.0L);
  for (int j = 0; j < n; ++j) {
    b[j] = std::conj(out.chirp[j]);
    if (j > 0) b[m - j] = std::conj(out.chirp[j]);
  }
  // B = DFT_m(b) / m, stored at the digit-reversed slots of the core DIF
  std::vector<std::complex<long double>> W(m);
  for (int k = 0; k < m; ++k) W[k] = root(k, m);
  out.bhat.assign(m, 0.0L);
  for (int k = 0; k < m; ++k) {
    std::complex<long double> s = 0.0L;
    long long idx = 0;
    for (int j = 0; j < m; ++j) {
      s += b[j] * W[idx];
      idx += k;
      if (idx >= m) idx -= m;
    }
    out.bhat[dif_slot(k, m, rad)] = s / (long double)m;
  }
  out.pos.resize(n);
  for (int k = 0; k < n; ++k) out.pos[k] = k;
  return true;
}

}  // namespace fhp
