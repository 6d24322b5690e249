// Engine<R>: device buffers, launch configuration and the call sequences of
// the operator, CG, energy and spectral interpolation.  Instantiated for
// double (fhp_engine_f64.cu) and float (fhp_engine_f32.cu).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fhp_engine.h"
#include "fhp_kernels.cuh"

namespace fhp {
// cuTensorMapEncodeTiled, looked up once through the runtime (no link to the
// driver library); null when the driver does not provide it
using TmapEncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline TmapEncodeFn tmap_encoder() {
  static TmapEncodeFn fn = []() -> TmapEncodeFn {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<TmapEncodeFn>(f);
  }();
  return fn;
}
// a 2D map of rows of `inner` 8-byte elements (row pitch inner * 8 bytes), box
// of one whole row; false if the driver rejects it
inline bool tmap_rows(CUtensorMap* m, void* base, unsigned long long inner,
                      unsigned long long rows) {
  TmapEncodeFn enc = tmap_encoder();
  if (!enc || inner > 256 || (inner * 8) % 16 != 0) return false;
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {inner * 8};
  const cuuint32_t box[2] = {(cuuint32_t)inner, 1};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace fhp

namespace fhp {

#define FHP_CHECK(call)                                                              \
  do {                                                                               \
    cudaError_t _e = (call);                                                         \
    if (_e != cudaSuccess) {                                                         \
      set_error(std::string("CUDA error: ") + cudaGetErrorString(_e) + " at " +     \
                __FILE__ + ":" + std::to_string(__LINE__));                          \
      return _e == cudaErrorMemoryAllocation ? ST_OOM : ST_CUDA;                     \
    }                                                                                \
  } while (0)

#define FHP_LAUNCHED()                                                               \
  do {                                                                               \
    ++launches;                                                                      \
    cudaError_t _e = cudaGetLastError();                                             \
    if (_e != cudaSuccess) {                                                         \
      set_error(std::string("kernel launch: ") + cudaGetErrorString(_e) + " at " +  \
                __FILE__ + ":" + std::to_string(__LINE__));                          \
      return ST_CUDA;                                                                \
    }                                                                                \
  } while (0)

constexpr int kThreads = 256;
constexpr size_t kSmemBudget = 96 * 1024;   // two CTAs per SM
constexpr size_t kSmemMax = 227 * 1024;
constexpr int kTargetElems = 8192;          // complex elements per CTA
// k_band_last per-CTA shared memory (lines + staged inputs): two CTAs per SM
// for FP32, one for FP64 (whose kernels use the full register file)
constexpr size_t kBandLastBudget32 = 110 * 1024;
// r2c / c2r last-axis passes: pair lines + staged c2r input, same split
constexpr size_t kRowBudget32 = 110 * 1024;
constexpr size_t kRowBudget64 = 220 * 1024;
constexpr size_t kBandLastBudget64 = 220 * 1024;

template <typename T>
static int set_smem_attr(T* kernel) {
  cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmemMax);
  if (e != cudaSuccess) {
    set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    return ST_CUDA;
  }
  return ST_OK;
}

template <typename R>
struct DevLine {
  LineDev<R> dev{};
  void* mem = nullptr;
};

template <typename R>
class Engine final : public EngineBase {
 public:
  explicit Engine(const PlanConfig& cfg) : cfg_(cfg) {}
  ~Engine() override { release(); }

  int init() {
    const int d = cfg_.dim;
    if (d != 2 && d != 3) { set_error("dim must be 2 or 3"); return ST_BAD_ARG; }
    for (int i = 0; i < d; ++i)
      if (cfg_.N[i] < 1 || cfg_.band[i] < 1 || !(cfg_.Y[i] > 0)) {
        set_error("grid sizes and cell lengths must be positive");
        return ST_BAD_ARG;
      }
    g_.dim = d;
    g_.n0 = d == 3 ? cfg_.N[0] : 1;
    g_.n1 = cfg_.N[d - 2];
    g_.n2 = cfg_.N[d - 1];
    g_.n2h = g_.n2 / 2 + 1;
    g_.dv = cfg_.physics == 0 ? d : cfg_.physics == 1 ? d * (d + 1) / 2 : cfg_.ncomp;
    g_.L = cfg_.nloads;
    set_grid_divs(g_);
    if (cfg_.physics < 0 && (g_.dv < 1 || g_.dv > kMaxDv)) {
      set_error("ncomp must be in 1..6");
      return ST_BAD_ARG;
    }
    if (g_.L < 1 || g_.L > kMaxLoads) { set_error("nloads must be in 1..6"); return ST_BAD_ARG; }
    g_.M = (long long)g_.n0 * g_.n1 * g_.n2;
    // cells of a batched plan: the grid's instance dimension (y or z, at most
    // 65535); band plans hold one cell
    g_.K = cfg_.ninst;
    if (g_.K < 1 || g_.K > 65535) { set_error("cells must be in 1..65535"); return ST_BAD_ARG; }
    if (g_.K > 1 && (cfg_.integ[0] > 0 || cfg_.physics < 0)) {
      set_error("batched plans hold GaNi or full-grid Ga cells");
      return ST_BAD_ARG;
    }
    gp_.physics = cfg_.physics;
    gp_.scale = cfg_.scale;
    for (int i = 0; i < 3; ++i) {
      const int b = i < d ? cfg_.band[i] : 1;
      const int bodd = b - ((b + 1) % 2);
      gp_.h[i] = (bodd - 1) / 2;
      gp_.Y[i] = i < d ? cfg_.Y[i] : 1.0;
      gp_.invY[i] = 1.0 / gp_.Y[i];
    }
    int st;
    if ((st = make_line(g_.n2, l2_)) != ST_OK) return st;
    if ((st = make_line(g_.n1, l1_)) != ST_OK) return st;
    if (d == 3 && (st = make_line(g_.n0, l0_)) != ST_OK) return st;
    const int C = g_.L * g_.dv;
    g_.sf = (long long)C * g_.M;
    g_.ss = (long long)C * g_.n0 * g_.n1 * g_.n2h;
    spec_elems_ = (size_t)g_.K * g_.ss;
    FHP_CHECK(cudaMalloc(&S_, spec_elems_ * sizeof(cplx<R>)));
    int dev = 0;
    FHP_CHECK(cudaGetDevice(&dev));
    FHP_CHECK(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev));
    // launch geometry
    const int np = (C + 1) / 2;
    // rows per CTA for the last-axis passes: pair lines plus (when it fits
    // the per-CTA budget) a staging area for the c2r input spectra; on small
    // grids fewer rows, so that the passes still spread over the SMs
    rows_ = set_row_geometry(std::min(std::max(1, kTargetElems / (np * l2_.dev.ld)),
                                      small_grid_cap((long long)g_.n0 * g_.n1)));
    if (smem_rows_ > kSmemMax) { set_error("line too long for shared memory"); return ST_BAD_ARG; }
    // strided c2c on axis 1 (3D) and projection on the first real axis
    if (d == 3) {
      // column passes: twice the line target (as the band-axis passes) fills
      // the radix stages of short lines and lengthens the contiguous rows
      T1_ = tile_cols(l1_.dev.ld, 1, (long long)g_.n2h, 2 * kTargetElems);
      T1_ = std::min(T1_, small_grid_cap((long long)g_.n2h * C * g_.n0, true));
    }
    const LineDev<R>& lp = (d == 3) ? l0_.dev : l1_.dev;
    const long long pin = (d == 3) ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    Tp_ = tile_cols(lp.ld, g_.dv, pin);
    Tp_ = std::min(Tp_, small_grid_cap(pin * g_.L, true));
    if ((size_t)Tp_ * g_.dv * lp.ld * sizeof(cplx<R>) > kSmemMax) {
      set_error("projection line too long for shared memory");
      return ST_BAD_ARG;
    }
    if (d == 3) T0_ = tile_cols(l0_.dev.ld, 1, (long long)g_.n1 * g_.n2h, 2 * kTargetElems);
    if (d == 3)
      T0_ = std::min(T0_, small_grid_cap((long long)g_.n1 * g_.n2h * C, true));
    if (cfg_.integ[0] > 0) {
      if ((st = init_band()) != ST_OK) return st;
    }
    // reduction scratch
    red_ctas_ = (int)std::max<long long>(1, std::min<long long>(4LL * nsm_, (g_.M + kThreads - 1) / kThreads));
    // parts of the reductions: row passes, grid-stride kernels, and the
    // component-split CG update (at least one part per component)
    nparts_max_ = std::max(std::max(row_ctas_, red_ctas_), g_.L * g_.dv);
    // per cell: partial sums, load states, reduced sums and per-load scales
    const size_t K = (size_t)g_.K;
    FHP_CHECK(cudaMalloc(&partials_,
                         K * nparts_max_ * kMaxLoads * kMaxLoads * sizeof(double)));
    FHP_CHECK(cudaMalloc(&st_, K * kMaxLoads * sizeof(LoadState)));
    FHP_CHECK(cudaMalloc(&all_done_, sizeof(int)));
    FHP_CHECK(cudaMallocHost(&h_done_, sizeof(int)));
    FHP_CHECK(cudaMalloc(&err_, sizeof(int)));
    FHP_CHECK(cudaMemset(err_, 0, sizeof(int)));
    FHP_CHECK(cudaMallocHost(&h_err_, sizeof(int)));
    FHP_CHECK(cudaMallocHost(&h_st_, K * kMaxLoads * sizeof(LoadState)));
    FHP_CHECK(cudaMalloc(&ad_, K * 2 * kMaxLoads * kMaxLoads * sizeof(double)));
    FHP_CHECK(cudaMalloc(&dscale_, K * 2 * kMaxLoads * sizeof(double)));
    return set_attrs();
  }

  int init_band() {
    const int d = cfg_.dim;
    band_ = true;
    gi_ = g_;
    gi_.n0 = d == 3 ? cfg_.integ[0] : 1;
    gi_.n1 = cfg_.integ[d - 2];
    gi_.n2 = cfg_.integ[d - 1];
    gi_.n2h = gi_.n2 / 2 + 1;
    gi_.M = (long long)gi_.n0 * gi_.n1 * gi_.n2;
    set_grid_divs(gi_);
    if (gi_.n0 < g_.n0 || gi_.n1 < g_.n1 || gi_.n2 < g_.n2) {
      set_error("integration grid must not be smaller than the solve grid");
      return ST_BAD_ARG;
    }
    double pb = (double)gi_.M;
    gp_.scale = cfg_.scale / pb;   // s / prod(B): normalised band coefficients
    int st;
    if ((st = make_line(gi_.n2, lb2_)) != ST_OK) return st;
    if ((st = make_line(gi_.n1, lb1_)) != ST_OK) return st;
    if (d == 3 && (st = make_line(gi_.n0, lb0_)) != ST_OK) return st;
    const int C = g_.L * g_.dv;
    const size_t n2h = (size_t)g_.n2h;
    const size_t sa = std::max((size_t)C * g_.n0 * g_.n1 * n2h, (size_t)C * gi_.n0 * gi_.n1 * n2h);
    const size_t sb = std::max((size_t)C * g_.n0 * gi_.n1 * n2h, (size_t)C * gi_.n0 * g_.n1 * n2h);
    cudaFree(S_);
    S_ = nullptr;
    spec_elems_ = sa;
    FHP_CHECK(cudaMalloc(&S_, sa * sizeof(cplx<R>)));
    FHP_CHECK(cudaMalloc(&SB_, sb * sizeof(cplx<R>)));
    const int np = (C + 1) / 2;
    const size_t srow = (size_t)np * lb2_.dev.ld * sizeof(cplx<R>);
    brows_ = std::max(1, kTargetElems / (np * lb2_.dev.ld));
    brows_ = (int)std::min<size_t>(brows_, std::max<size_t>(1, kSmemBudget / srow));
    bsmem_rows_ = (size_t)brows_ * srow;
    if (bsmem_rows_ > kSmemMax) { set_error("integration line too long"); return ST_BAD_ARG; }
    brow_ctas_ = (int)(((long long)gi_.n0 * gi_.n1 + brows_ - 1) / brows_);
    return ST_OK;
  }

  // rows per CTA of the last-axis passes: pair lines plus (when it fits the
  // per-CTA budget) a staging area for the c2r input spectra; the request is
  // reduced until it fits.  Sets rows_, c2r_stage_, smem_rows_, row_ctas_.
  // Largest rows (columns) per CTA that still give about two CTAs per SM when
  // a pass has `units` rows (columns) per cell: small grids spread over the
  // SMs instead of running a few long CTAs (a power of two for column tiles).
  // Per cell, so a plan of several cells computes each cell as a plan of that
  // cell alone does.
  int small_grid_cap(long long units, bool pow2 = false) const {
    long long c = std::max<long long>(1, units / (2LL * std::max(1, nsm_)));
    c = std::min<long long>(c, 1 << 20);
    int r = (int)c;
    if (pow2)
      while (r & (r - 1)) r &= r - 1;
    return std::max(1, r);
  }

  int set_row_geometry(int want) {
    const int C = g_.L * g_.dv, np = (C + 1) / 2;
    const size_t srow = (size_t)np * l2_.dev.ld * sizeof(cplx<R>);
    const size_t sraw_row = (size_t)C * g_.n2h * sizeof(cplx<R>);
    const size_t budget = sizeof(R) == 4 ? kRowBudget32 : kRowBudget64;
    auto smem_of = [&](int r, bool stg) {
      return align16((size_t)r * srow) + (stg ? (size_t)r * sraw_row : 0);
    };
    int r = std::max(1, want);
    c2r_stage_ = smem_of(1, true) <= budget;
    while (r > 1 && smem_of(r, c2r_stage_) > budget) --r;
    rows_ = r;
    smem_rows_ = std::max<size_t>(smem_of(r, c2r_stage_), 8 * kMaxLoads * sizeof(double));
    row_ctas_ = (int)(((long long)g_.n0 * g_.n1 + r - 1) / r);
    return r;
  }

  // ---- autotuning: launch shapes timed on this plan's own buffers ----------
  // Candidates: band plans - the integration kernel (register lines with 1 or
  // 2 CTAs per SM where they apply, or the shared-memory cores) and the
  // column-tile target of the axis passes (1x, 2x, 4x the line target);
  // other plans - rows per CTA of the last-axis passes and the column tile of
  // the first-axis projection pass.  Each candidate is timed over three
  // operator applications (CUDA events, after one warm-up) and the fastest
  // is kept; the choice is cached per plan geometry, precision, coefficient
  // kind and device, so plans of the same shape reuse it.
  struct TuneChoice { int a = 0, b = 0, c = 0; float ms = 0.f; };
  static std::mutex& tune_mu() { static std::mutex m; return m; }
  static std::map<std::string, TuneChoice>& tune_cache() {
    static std::map<std::string, TuneChoice> c;
    return c;
  }
  std::string tune_key() const {
    int dev = 0;
    cudaGetDevice(&dev);
    std::string k = std::to_string(dev) + (sizeof(R) == 8 ? ":f64" : ":f32") + ":d" +
                    std::to_string(g_.dim) + ":p" + std::to_string(cfg_.physics) + ":L" +
                    std::to_string(g_.L) + ":k" + std::to_string(coef_kind_) + ":K" +
                    std::to_string(g_.K);
    for (int i = 0; i < 3; ++i) k += ":" + std::to_string(cfg_.N[i]) + "/" + std::to_string(cfg_.integ[i]);
    return k;
  }
  void tune_apply(const TuneChoice& c) {
    if (band_) {
      integ_kernel_ = c.a;
      if (c.a == 1) reg512_ctas_per_sm_ = c.b;
      axis_target_mult_ = c.c;
    } else {
      set_row_geometry(c.a);
      Tp_ = c.b;
    }
  }
  int autotune(cudaStream_t s, int* chosen, float* best_ms) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    const std::string key = tune_key();
    {
      std::lock_guard<std::mutex> g(tune_mu());
      auto it = tune_cache().find(key);
      if (it != tune_cache().end()) {
        tune_apply(it->second);
        if (chosen) { chosen[0] = it->second.a; chosen[1] = it->second.b; chosen[2] = it->second.c; }
        if (best_ms) *best_ms = it->second.ms;
        return ST_OK;
      }
    }
    std::vector<TuneChoice> cand;
    if (band_) {
      for (int m : {1, 2, 4}) {
        if (reg512_applies(coef_kind_)) {
          cand.push_back({1, 1, m});
          cand.push_back({1, 2, m});
        }
        cand.push_back({0, 0, m});
      }
    } else {
      const int d = g_.dim;
      const LineDev<R>& lp = d == 3 ? l0_.dev : l1_.dev;
      const long long pin = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
      for (int r : {1, 2, 4, 8, 16, 32}) {
        if (r > 1 && r > g_.n0 * g_.n1) break;
        for (int T = 1; T <= 32 && T <= pin; T *= 2) {
          if ((size_t)T * g_.dv * lp.ld * sizeof(cplx<R>) > kSmemMax) break;
          cand.push_back({r, T, 0});
        }
      }
    }
    // partial sums must hold the most CTAs any candidate launches
    const int save_rows = rows_, save_Tp = Tp_, save_ik = integ_kernel_,
              save_rc = reg512_ctas_per_sm_, save_m = axis_target_mult_;
    int st = ensure_cg_buffers();
    if (st != ST_OK) return st;
    {
      const long long worst = ((long long)g_.n0 * g_.n1);
      if (worst > nparts_max_) {
        double* np = nullptr;
        FHP_CHECK(cudaMalloc(&np, (size_t)g_.K * worst * kMaxLoads * kMaxLoads * sizeof(double)));
        cudaFree(partials_);
        partials_ = np;
        nparts_max_ = (int)worst;
      }
    }
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    k_fill_macro<R><<<grid_for(n), kThreads, 0, s>>>(r_, g_, 1.0);
    FHP_LAUNCHED();
    cudaEvent_t e0, e1;
    FHP_CHECK(cudaEventCreate(&e0));
    FHP_CHECK(cudaEventCreate(&e1));
    TuneChoice best;
    best.ms = 1e30f;
    for (const TuneChoice& c : cand) {
      tune_apply(c);
      if ((st = apply_ex(1, r_, ap_, s, false)) != ST_OK) break;
      cudaEventRecord(e0, s);
      for (int rep = 0; rep < 3 && st == ST_OK; ++rep) st = apply_ex(1, r_, ap_, s, false);
      cudaEventRecord(e1, s);
      if (st != ST_OK || cudaEventSynchronize(e1) != cudaSuccess) { st = st ? st : ST_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best.ms) { best = c; best.ms = ms; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != ST_OK || cand.empty()) {
      rows_ = save_rows;
      set_row_geometry(save_rows);
      Tp_ = save_Tp;
      integ_kernel_ = save_ik;
      reg512_ctas_per_sm_ = save_rc;
      axis_target_mult_ = save_m;
      return st;
    }
    best.ms /= 3.f;
    tune_apply(best);
    {
      std::lock_guard<std::mutex> g(tune_mu());
      tune_cache()[key] = best;
    }
    if (chosen) { chosen[0] = best.a; chosen[1] = best.b; chosen[2] = best.c; }
    if (best_ms) *best_ms = best.ms;
    return ST_OK;
  }

  int precision() const override { return sizeof(R) == 8 ? 0 : 1; }
  long long voxels() const override { return g_.M; }
  int dv() const override { return g_.dv; }
  int loads() const override { return g_.L; }
  int instances() const override { return g_.K; }
  long long coef_voxels() const override { return band_ ? gi_.M : g_.M; }
  void set_load_tols(const double* tols, int n) override { load_tol_.assign(tols, tols + n); }
  size_t elem_size() const override { return sizeof(R); }
  size_t spectrum_elems() const override { return spec_elems_; }
  const PlanConfig& config() const override { return cfg_; }
  int coef_kind() const override { return coef_kind_; }

  // ---- potential formulation (homogenisation.py:41-127) --------------------
  long long pot_spectrum_elems() const override {
    const int d = g_.dim;
    const long long b0 = d == 3 ? cfg_.band[0] : 1, b1 = cfg_.band[d - 2], b2 = cfg_.band[d - 1];
    return (long long)g_.L * b0 * b1 * (b2 / 2 + 1);
  }

  int pot_check() {
    if (cfg_.physics != 0) { set_error("the potential formulation is scalar"); return ST_BAD_ARG; }
    if (band_) {
      set_error("the potential formulation needs a plan without an integration grid");
      return ST_BAD_ARG;
    }
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    const int d = g_.dim;
    const int ns[3] = {g_.n0, g_.n1, g_.n2};
    for (int a = 0; a < d; ++a) {
      const int n = cfg_.band[a], gs = ns[3 - d + a];
      if (gs != n && (n % 2 == 0 || gs < n)) {
        set_error("potential formulation: a grid larger than the potential grid needs odd N");
        return ST_BAD_ARG;
      }
    }
    PotParams& pp = pp_;
    pp.nb[0] = d == 3 ? cfg_.band[0] : 1;
    pp.nb[1] = cfg_.band[d - 2];
    pp.nb[2] = cfg_.band[d - 1];
    pp.nbh = pp.nb[2] / 2 + 1;
    pp.Yg[0] = d == 3 ? cfg_.Y[0] : 1.0;
    pp.Yg[1] = cfg_.Y[d - 2];
    pp.Yg[2] = cfg_.Y[d - 1];
    pp.scale = (double)g_.M / ((double)pp.nb[0] * pp.nb[1] * pp.nb[2]);
    pp.zs = 1.0 / ((double)pp.nb[0] * pp.nb[1] * pp.nb[2]);
    for (int a = 0; a < 3; ++a) {
      pp.tpy[a] = 6.283185307179586476925286766559 / pp.Yg[a];
      pp.tpy_f[a] = (float)pp.tpy[a];
    }
    pp.izs = 1.0 / pp.zs;
    pp.iscale = 1.0 / pp.scale;
    pp.scale_f = (float)pp.scale;
    pp.zs_f = (float)pp.zs;
    pp.izs_f = (float)pp.izs;
    pp.iscale_f = (float)pp.iscale;
    if (!pe_) {
      FHP_CHECK(cudaMalloc(&pe_, (size_t)g_.K * g_.L * g_.dv * g_.M * sizeof(R)));
      const int T = d == 3 ? T0_ : tile_cols(l1_.dev.ld, 1, (long long)g_.n2h);
      Tfirst_ = T;
    }
    return ST_OK;
  }

  // full inverse transform of S_ into the fields y (1/M)
  int pot_inv(R* y, bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const LoadState* st = cg ? st_ : nullptr;
    const int d = g_.dim;
    const DevLine<R>& lf = d == 3 ? l0_ : l1_;
    const long long inner = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    dim3 grid((unsigned)((inner + Tfirst_ - 1) / Tfirst_), (unsigned)(g_.L * g_.dv));
    const int pk = pbeg("pot_c2c_first_inv", 2.0 * spec_bytes(), s);
    k_c2c_axis<R, true><<<grid, kThreads, (size_t)Tfirst_ * lf.dev.ld * sizeof(cplx<R>), s>>>(
        S_, d == 3 ? g_.n0 : g_.n1, inner, lf.dev, Tfirst_, ad, st, g_.dv, g_.ss, g_.L);
    pend(pk, s);
    FHP_LAUNCHED();
    return inv_passes(S_, y, (R)(1.0 / (double)g_.M), false, nullptr, cg, s);
  }

  // full forward transform of A x into S_
  int pot_fwd(const R* x, bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const LoadState* st = cg ? st_ : nullptr;
    int rc = fwd_passes(coef_kind_, false, x, nullptr, nullptr, S_, cg, s);
    if (rc != ST_OK) return rc;
    const int d = g_.dim;
    const DevLine<R>& lf = d == 3 ? l0_ : l1_;
    const long long inner = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    dim3 grid((unsigned)((inner + Tfirst_ - 1) / Tfirst_), (unsigned)(g_.L * g_.dv));
    const int pk = pbeg("pot_c2c_first_fwd", 2.0 * spec_bytes(), s);
    k_c2c_axis<R, false><<<grid, kThreads, (size_t)Tfirst_ * lf.dev.ld * sizeof(cplx<R>), s>>>(
        S_, d == 3 ? g_.n0 : g_.n1, inner, lf.dev, Tfirst_, ad, st, g_.dv, g_.ss, g_.L);
    pend(pk, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // y = P (-div) decrease F A iF enlarge grad P x ; zio: x and y z-scaled
  int pot_operator(const cplx<R>* x, cplx<R>* y, bool zio, bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const long long ns = (long long)g_.n0 * g_.n1 * g_.n2h;
    const int pke = pbeg("pot_expand", (double)pot_spectrum_elems() * sizeof(cplx<R>) +
                                           g_.dim * spec_bytes() / g_.dv, s);
    k_pot_expand<R><<<dim3(grid_for((size_t)ns), g_.L), kThreads, 0, s>>>(x, S_, g_, pp_,
                                                                        zio ? 1 : 0, ad);
    pend(pke, s);
    FHP_LAUNCHED();
    int rc = pot_inv(pe_, cg, s);
    if (rc == ST_OK) rc = pot_fwd(pe_, cg, s);
    if (rc != ST_OK) return rc;
    const int pkc = pbeg("pot_contract", (double)pot_spectrum_elems() * sizeof(cplx<R>) +
                                             g_.dim * spec_bytes() / g_.dv, s);
    k_pot_contract<R><<<dim3(grid_for((size_t)(pot_spectrum_elems() / g_.L)), g_.L), kThreads,
                        0, s>>>(S_, y, g_, pp_, -1.0, zio ? 1 : 0, ad);
    pend(pkc, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int pot_rhs(void* bh, cudaStream_t s) override {
    int rc = pot_check();
    if (rc != ST_OK) return rc;
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    k_fill_macro<R><<<grid_for(n), kThreads, 0, s>>>(pe_, g_, 1.0);
    FHP_LAUNCHED();
    if ((rc = pot_fwd(pe_, false, s)) != ST_OK) return rc;
    k_pot_contract<R><<<dim3(grid_for((size_t)(pot_spectrum_elems() / g_.L)), g_.L), kThreads,
                        0, s>>>(S_, static_cast<cplx<R>*>(bh), g_, pp_, 1.0, 0, nullptr);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int pot_apply(const void* xh, void* yh, cudaStream_t s) override {
    int rc = pot_check();
    if (rc != ST_OK) return rc;
    return pot_operator(static_cast<const cplx<R>*>(xh), static_cast<cplx<R>*>(yh), false,
                        false, s);
  }

  int pot_field(const void* xh, void* X, cudaStream_t s) override {
    int rc = pot_check();
    if (rc != ST_OK) return rc;
    const long long ns = (long long)g_.n0 * g_.n1 * g_.n2h;
    k_pot_expand<R><<<dim3(grid_for((size_t)ns), g_.L), kThreads, 0, s>>>(
        static_cast<const cplx<R>*>(xh), S_, g_, pp_, 0, nullptr);
    FHP_LAUNCHED();
    return pot_inv(static_cast<R*>(X), false, s);
  }

  // CG (solver.py:80-139) in z = sqrt(w) x / prod(N): the 'r' inner product
  // (objects.py:618-631) is the Euclidean one of z, so the field CG kernels
  // run on the z vectors (2 prod(N0 N1 (N2/2+1)) reals per load) with a
  // unit mean factor.  x0 = 0 (homogenisation.py:59, 96).
  int pot_cg(const void* bh, double tol, int maxiter, void* xh, SolveResult& res, int log_cap,
             cudaStream_t s) override {
    int rc = pot_check();
    if (rc != ST_OK) return rc;
    const long long mz = pot_spectrum_elems() / g_.L;  // complex entries per load
    const size_t nz = (size_t)g_.L * mz;
    if (!zx_) {
      FHP_CHECK(cudaMalloc(&zx_, 4 * nz * sizeof(cplx<R>)));
    }
    cplx<R>* zx = zx_;
    cplx<R>* zr = zx_ + nz;
    cplx<R>* zp = zx_ + 2 * nz;
    cplx<R>* zap = zx_ + 3 * nz;
    GridDims gz = g_;
    gz.dv = 1;
    gz.M = 2 * mz;
    R* rx = reinterpret_cast<R*>(zx);
    R* rr = reinterpret_cast<R*>(zr);
    R* rp = reinterpret_cast<R*>(zp);
    R* rap = reinterpret_cast<R*>(zap);
    FHP_CHECK(cudaMemsetAsync(zx, 0, nz * sizeof(cplx<R>), s));
    k_pot_zscale<R><<<grid_for(nz), kThreads, 0, s>>>(static_cast<const cplx<R>*>(bh), zr,
                                                       (long long)nz, pp_, 1);
    FHP_LAUNCHED();
    FHP_CHECK(cudaMemcpyAsync(zp, zr, nz * sizeof(cplx<R>), cudaMemcpyDeviceToDevice, s));
    for (int l = 0; l < g_.L; ++l) {
      LoadState& h = h_st_[l];
      std::memset(&h, 0, sizeof(LoadState));
      h.tol = tol;
      h.maxiter = maxiter;
      h.guard = sizeof(R) == 4 ? 4.0 : 0.0;
    }
    FHP_CHECK(cudaMemcpyAsync(st_, h_st_, g_.L * sizeof(LoadState), cudaMemcpyHostToDevice, s));
    FHP_CHECK(cudaMemsetAsync(all_done_, 0, sizeof(int), s));
    const int log_rows = std::max(1, std::min(log_cap, maxiter + 1));
    double* dlog =
        static_cast<double*>(scratch(SCR_LOG, (size_t)log_rows * g_.L * sizeof(double)));
    if (!dlog) return ST_OOM;
    FHP_CHECK(cudaMemsetAsync(dlog, 0, (size_t)log_rows * g_.L * sizeof(double), s));
    k_dot<R><<<red_ctas_, kThreads, 0, s>>>(rr, rr, partials_, gz);
    FHP_LAUNCHED();
    k_fin_init<<<1, 32, 0, s>>>(partials_, red_ctas_, st_, g_.L, 1.0, dlog, log_rows);
    FHP_LAUNCHED();
    k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
    FHP_LAUNCHED();
    int done_iters = 0, chunk = 2;
    while (done_iters < maxiter) {
      FHP_CHECK(cudaMemcpyAsync(h_done_, all_done_, sizeof(int), cudaMemcpyDeviceToHost, s));
      FHP_CHECK(cudaStreamSynchronize(s));
      if (*h_done_) break;
      const int nit = std::min(chunk, maxiter - done_iters);
      for (int it = 0; it < nit && rc == ST_OK; ++it) {
        rc = pot_operator(zp, zap, true, true, s);
        if (rc != ST_OK) break;
        const double zb = (double)nz * sizeof(cplx<R>);   // one z vector
        int pk = pbeg("pot_dot", 2.0 * zb, s);
        k_dot<R><<<red_ctas_, kThreads, 0, s>>>(rp, rap, partials_, gz);
        pend(pk, s);
        FHP_LAUNCHED();
        k_fin_pap<<<g_.L, kThreads, 0, s>>>(partials_, red_ctas_, st_, g_.L, 1.0, all_done_);
        FHP_LAUNCHED();
        pk = pbeg("pot_cg_update", 6.0 * zb, s);
        k_cg_update<R><<<red_ctas_, kThreads, 0, s>>>(rx, rr, rp, rap, partials_, gz, st_,
                                                      all_done_);
        pend(pk, s);
        FHP_LAUNCHED();
        k_fin_rr<<<g_.L, kThreads, 0, s>>>(partials_, red_ctas_, st_, g_.L, 1.0, dlog, log_rows,
                                           all_done_);
        FHP_LAUNCHED();
        pk = pbeg("pot_p_update", 3.0 * zb, s);
        k_p_update<R><<<grid_for(2 * nz), kThreads, 0, s>>>(rr, rp, gz, st_, all_done_);
        pend(pk, s);
        FHP_LAUNCHED();
        k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
        FHP_LAUNCHED();
      }
      if (rc != ST_OK) break;
      done_iters += nit;
      chunk = std::min(chunk * 2, 32);
    }
    if (rc == ST_OK) {
      k_pot_zscale<R><<<grid_for(nz), kThreads, 0, s>>>(zx, static_cast<cplx<R>*>(xh),
                                                         (long long)nz, pp_, 0);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); rc = ST_CUDA; }
      ++launches;
    }
    if (rc != ST_OK) return rc;
    FHP_CHECK(cudaMemcpyAsync(h_st_, st_, g_.L * sizeof(LoadState), cudaMemcpyDeviceToHost, s));
    res.res_log.assign((size_t)log_rows * g_.L, 0.0);
    FHP_CHECK(cudaMemcpyAsync(res.res_log.data(), dlog, (size_t)log_rows * g_.L * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaStreamSynchronize(s));
    res.kit.resize(g_.L);
    res.norm_res.resize(g_.L);
    res.status.resize(g_.L);
    res.iterations_run = 0;
    for (int l = 0; l < g_.L; ++l) {
      const LoadState& h = h_st_[l];
      res.kit[l] = h.kit;
      res.norm_res[l] = h.kit == 0 ? 0.0 : h.norm_res;
      int sl = h.status;
      if (sl == 0 && h.norm_res > tol && h.kit > 0) sl = ST_NONCONVERGED;
      res.status[l] = sl;
      res.iterations_run = std::max(res.iterations_run, h.kit);
    }
    return ST_OK;
  }

  int set_coefficient(int kind, const double* values, bool on_device, cudaStream_t s) override {
    if (kind < COEF_ISO || kind > COEF_FULL) { set_error("bad coefficient kind"); return ST_BAD_ARG; }
    const int dv = g_.dv;
    const int c = kind == COEF_ISO ? 1 : kind == COEF_SYM ? dv * (dv + 1) / 2 : dv * dv;
    // [cell][c][grid]: every cell of a batched plan has its own coefficient
    const size_t n = (size_t)g_.K * c * (band_ ? gi_.M : g_.M);
    g_.sa = (long long)c * (band_ ? gi_.M : g_.M);
    // keep the buffer when it is large enough: cudaFree synchronises the device,
    // which would serialise plans working on other streams
    if (A_ && A_elems_ < n) { cudaFree(A_); A_ = nullptr; }
    if (!A_) {
      FHP_CHECK(cudaMalloc(&A_, n * sizeof(R)));
      A_elems_ = n;
    }
    // host values go through the plan's persistent staging buffer (no
    // allocation per call); the copy from pageable memory has read the host
    // buffer when the call returns
    double* tmp = nullptr;
    const double* src = values;
    if (!on_device) {
      tmp = static_cast<double*>(scratch(SCR_COEF_STAGE, n * sizeof(double)));
      if (!tmp) return ST_OOM;
      FHP_CHECK(cudaMemcpyAsync(tmp, values, n * sizeof(double), cudaMemcpyHostToDevice, s));
      src = tmp;
    }
    k_convert<R, double><<<grid_for(n), kThreads, 0, s>>>((long long)n, src, A_);
    FHP_LAUNCHED();
    coef_kind_ = kind;
    return ST_OK;
  }

  // y = iF G F (A x) for all loads (ffthompy/tensors/operators.py:136-144)
  int apply(int proj, const void* x, void* y, cudaStream_t s) override {
    return apply_ex(proj, x, y, s, false);
  }

  // inproj: G A G (band mode), see band_operator
  int apply_ex(int proj, const void* x, void* y, cudaStream_t s, bool inproj) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    gp_.proj = proj;
    return run_operator(coef_kind_, false, static_cast<const R*>(x), nullptr, nullptr,
                        static_cast<R*>(y), nullptr, s, false, false, inproj);
  }

  int axpy(double a, const void* x, void* y, cudaStream_t s) override {
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    k_axpby<R><<<grid_for(n), kThreads, 0, s>>>((long long)n, a, static_cast<const R*>(x), 1.0,
                                                static_cast<R*>(y));
    FHP_LAUNCHED();
    return ST_OK;
  }

  // y = G x (orthogonal projection onto the compatible / equilibrated fields
  // of the solve grid band)
  int project(int proj, const void* xv, void* yv, cudaStream_t s) override {
    const int proj_saved = gp_.proj;
    const double scale_saved = gp_.scale;
    gp_.proj = proj;
    gp_.scale = 1.0;
    int st = fwd_passes(COEF_NONE, false, static_cast<const R*>(xv), nullptr, nullptr, S_, false,
                        s);
    if (st == ST_OK) st = proj_pass(S_, false, s);
    if (st == ST_OK) st = inv_passes(S_, static_cast<R*>(yv), (R)(1.0 / (double)g_.M), false,
                                     nullptr, false, s);
    gp_.proj = proj_saved;
    gp_.scale = scale_saved;
    return st;
  }

  int rhs_macro(int proj, void* b, cudaStream_t s) override {
    if (band_ && spectral_cg_) return spectral_rhs(proj, static_cast<R*>(b), s);
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    R* tmp = static_cast<R*>(scratch(SCR_RHS_TMP, n * sizeof(R)));
    if (!tmp) return ST_OOM;
    k_fill_macro<R><<<grid_for(n), kThreads, 0, s>>>(tmp, g_, -1.0);
    FHP_LAUNCHED();
    return apply(proj, tmp, b, s);
  }

  int cg_solve(int proj, const void* bv, const void* x0v, double tol, int maxiter, void* xv,
               SolveResult& res, int log_cap, cudaStream_t s) override {
    int st = cg_begin(proj, bv, x0v, tol, maxiter, xv, log_cap, s);
    if (st != ST_OK) return st;
    st = iterate(maxiter, s, [&]() { return cg_step(s); });
    if (st != ST_OK) return st;
    return cg_end(res, s);
  }

  // ---- Richardson / Chebyshev / BiCG (solver.py:63-77, 142-285) -----------
  // The operator runs with the per-load done flags (done loads skipped), the
  // recurrences in fused component-row kernels with per-load scalars on the
  // device, one iteration per CUDA-graph replay, and the host reads the
  // all-done flag between chunks of iterations, as in cg_solve.
  int solve_other(int kind, int proj, const void* bv, const void* x0v, double p0, double p1,
                  double tol, int maxiter, void* xv, SolveResult& res, int log_cap,
                  cudaStream_t s) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    if (kind < 0 || kind > 2) { set_error("unknown solver"); return ST_BAD_ARG; }
    gp_.proj = proj;
    const R* b = static_cast<const R*>(bv);
    const R* x0 = static_cast<const R*>(x0v);
    R* x = static_cast<R*>(xv);
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    int st = ensure_cg_buffers();
    if (st != ST_OK) return st;
    R* va = static_cast<R*>(scratch(SCR_SOLV_A, n * sizeof(R)));
    R* vb = static_cast<R*>(scratch(SCR_SOLV_B, n * sizeof(R)));
    R* vc = static_cast<R*>(scratch(SCR_SOLV_C, n * sizeof(R)));
    if (!va || !vb || !vc) return ST_OOM;
    if (x0) FHP_CHECK(cudaMemcpyAsync(x, x0, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
    else FHP_CHECK(cudaMemsetAsync(x, 0, n * sizeof(R), s));
    if ((st = init_state(tol, maxiter, log_cap, s)) != ST_OK) return st;
    const double invM = 1.0 / (double)g_.M;
    const int C = g_.L * g_.dv;
    const int ux = std::max(1, red_ctas_ / C);
    const dim3 cgrid((unsigned)ux, (unsigned)C);
    auto op = [&](const R* in, R* out) {
      return run_operator(coef_kind_, false, in, nullptr, nullptr, out, nullptr, s, true, false);
    };
    auto sum_into = [&](double* dst_rr, bool relative) {
      // partials of a component-row kernel -> per-load norm (relative to r0)
      k_fin_norm<<<g_.L, kThreads, 0, s>>>(partials_, ux * C, st_, g_.L, invM,
                                           relative ? 1 : 0, cg_log_, cg_log_rows_, all_done_);
      (void)dst_rr;
    };
    std::function<int()> step;
    if (kind == 0) {
      // norm_res starts at 1e15 (solver.py:65-66): the first iteration runs
      k_set_norm<<<1, 32, 0, s>>>(st_, g_.L, 1e15);
      FHP_LAUNCHED();
      step = [&, b, x]() -> int {
        int r = op(x, ap_);
        if (r != ST_OK) return r;
        k_resid_comp<R, 0><<<cgrid, kThreads, 0, s>>>(b, ap_, x, p0, partials_, g_, st_,
                                                     all_done_);
        FHP_LAUNCHED();
        sum_into(nullptr, false);
        FHP_LAUNCHED();
        k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
        FHP_LAUNCHED();
        return ST_OK;
      };
    } else if (kind == 1) {
      // r = B - A x0, r0 = |r| (pap), norm_res = r0 / |B| (solver.py:226-236)
      if ((st = op(x, ap_)) != ST_OK) return st;
      k_resid_comp<R, 1><<<cgrid, kThreads, 0, s>>>(b, ap_, r_, 0., partials_, g_, st_, nullptr);
      FHP_LAUNCHED();
      k_dot<R><<<red_ctas_, kThreads, 0, s>>>(b, b, partials_ + (size_t)ux * C * g_.L, g_);
      FHP_LAUNCHED();
      k_cheb_init<<<1, 32, 0, s>>>(partials_, ux * C, partials_ + (size_t)ux * C * g_.L,
                                   red_ctas_, st_, g_.L, invM, cg_log_, cg_log_rows_);
      FHP_LAUNCHED();
      k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
      FHP_LAUNCHED();
      FHP_CHECK(cudaMemsetAsync(va, 0, n * sizeof(R), s));  // v = 0
      const double d = (p1 + p0) / 2.0, c = (p1 - p0) / 2.0;
      step = [&, b, x, va, d, c]() -> int {
        k_cheb_coef<<<1, 32, 0, s>>>(st_, g_.L, d, c, all_done_);
        FHP_LAUNCHED();
        k_cheb_update<R><<<cgrid, kThreads, 0, s>>>(r_, va, x, g_, st_, all_done_);
        FHP_LAUNCHED();
        int r = op(x, ap_);
        if (r != ST_OK) return r;
        k_resid_comp<R, 1><<<cgrid, kThreads, 0, s>>>(b, ap_, r_, 0., partials_, g_, st_,
                                                     all_done_);
        FHP_LAUNCHED();
        sum_into(nullptr, true);
        FHP_LAUNCHED();
        k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
        FHP_LAUNCHED();
        return ST_OK;
      };
    } else {
      // R = B - A x0, Rs = R, P = R, Ps = Rs, rr = <R, Rs> (solver.py:158-166)
      R* rs = va;
      R* ps = vb;
      R* atps = vc;
      if ((st = op(x, ap_)) != ST_OK) return st;
      FHP_CHECK(cudaMemcpyAsync(r_, b, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      k_axpby<R><<<grid_for(n), kThreads, 0, s>>>((long long)n, -1.0, ap_, 1.0, r_);
      FHP_LAUNCHED();
      FHP_CHECK(cudaMemcpyAsync(rs, r_, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      FHP_CHECK(cudaMemcpyAsync(p_, r_, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      FHP_CHECK(cudaMemcpyAsync(ps, r_, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      k_dot<R><<<red_ctas_, kThreads, 0, s>>>(r_, rs, partials_, g_);
      FHP_LAUNCHED();
      k_fin_init<<<1, 32, 0, s>>>(partials_, red_ctas_, st_, g_.L, invM, cg_log_, cg_log_rows_);
      FHP_LAUNCHED();
      k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
      FHP_LAUNCHED();
      step = [&, x, rs, ps, atps]() -> int {
        int r = op(p_, ap_);
        if (r == ST_OK) r = op(ps, atps);
        if (r != ST_OK) return r;
        k_dot<R><<<red_ctas_, kThreads, 0, s>>>(ap_, ps, partials_, g_);
        FHP_LAUNCHED();
        k_fin_pap<<<g_.L, kThreads, 0, s>>>(partials_, red_ctas_, st_, g_.L, invM, all_done_);
        FHP_LAUNCHED();
        k_bicg_update<R><<<cgrid, kThreads, 0, s>>>(x, r_, rs, p_, ap_, atps, partials_, g_, st_,
                                                    all_done_);
        FHP_LAUNCHED();
        k_fin_rr<<<g_.L, kThreads, 0, s>>>(partials_, ux * C, st_, g_.L, invM, cg_log_,
                                           cg_log_rows_, all_done_);
        FHP_LAUNCHED();
        k_bicg_dirs<R><<<cgrid, kThreads, 0, s>>>(r_, rs, p_, ps, g_, st_, all_done_);
        FHP_LAUNCHED();
        k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
        FHP_LAUNCHED();
        return ST_OK;
      };
    }
    if ((st = iterate(maxiter, s, step)) != ST_OK) return st;
    if ((st = collect(tol, cg_log_rows_, cg_log_, res, s)) != ST_OK) return st;
    // Chebyshev returns at once with norm_res = r0 / |B| when that is below
    // tol (solver.py:234-236)
    if (kind == 1)
      for (int l = 0; l < g_.L; ++l)
        if (res.kit[l] == 0 && h_st_[l].norm_res < tol) res.norm_res[l] = h_st_[l].norm_res;
    return ST_OK;
  }

  // ---- CG in phases: begin (state, first residual), step (one iteration's
  // launches, capturable), end (final projection, results).  cg_solve runs
  // them for one plan; fhp_cg_solve_many advances several plans together.
  int cg_begin(int proj, const void* bv, const void* x0v, double tol, int maxiter, void* xv,
               int log_cap, cudaStream_t s) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    gp_.proj = proj;
    const R* b = static_cast<const R*>(bv);
    const R* x0 = static_cast<const R*>(x0v);
    R* x = static_cast<R*>(xv);
    cg_spectral_ = band_ && spectral_cg_;
    cg_proj_ = proj;
    cg_tol_ = tol;
    cg_x_ = x;
    if (cg_spectral_) return spectral_cg_begin(proj, b, x0, tol, maxiter, log_cap, s);
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    int st = ensure_cg_buffers();
    if (st != ST_OK) return st;
    // x = x0 ; R = B - A x0 ; P = R   (solver.py:114-117)
    if (x0) {
      FHP_CHECK(cudaMemcpyAsync(x, x0, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      if ((st = apply_ex(proj, x, ap_, s, true)) != ST_OK) return st;
      FHP_CHECK(cudaMemcpyAsync(r_, b, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      k_axpby<R><<<grid_for(n), kThreads, 0, s>>>((long long)n, -1.0, ap_, 1.0, r_);
      FHP_LAUNCHED();
    } else {
      FHP_CHECK(cudaMemsetAsync(x, 0, n * sizeof(R), s));
      FHP_CHECK(cudaMemcpyAsync(r_, b, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
    }
    FHP_CHECK(cudaMemcpyAsync(p_, r_, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
    x_cur_ = x;
    if ((st = init_state(tol, maxiter, log_cap, s)) != ST_OK) return st;
    k_dot<R><<<dim3(red_ctas_, g_.K), kThreads, 0, s>>>(r_, r_, partials_, g_);
    FHP_LAUNCHED();
    k_fin_init<<<g_.K, 32, 0, s>>>(partials_, red_ctas_, st_, g_.L, 1.0 / (double)g_.M, cg_log_,
                                   cg_log_rows_);
    FHP_LAUNCHED();
    k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L * g_.K, all_done_);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int cg_step(cudaStream_t s) override {
    if (cg_spectral_) {
      const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
      return spectral_iteration(zb_, zb_ + nz, zb_ + 2 * nz, zb_ + 3 * nz, cg_log_, cg_log_rows_,
                                s);
    }
    return cg_iteration(cg_log_, cg_log_rows_, s);
  }

  const int* cg_done_flag() const override { return all_done_; }

  int cg_end(SolveResult& res, cudaStream_t s) override {
    int st;
    if (cg_spectral_) {
      // back to the caller's real field; FP32 iterates are projected first
      // (roundoff of the updates outside range(G))
      if (sizeof(R) == 4 && (st = spec_green(zb_, s)) != ST_OK) return st;
      if ((st = from_z(zb_, cg_x_, s)) != ST_OK) return st;
    } else if (sizeof(R) == 4 && (st = project(cg_proj_, cg_x_, cg_x_, s)) != ST_OK) {
      // FP32 fields: the iterate drifts out of range(G) by roundoff accumulated
      // over the iterations, and that component enters the energy to first
      // order. One projection x <- G x (the identity in exact arithmetic) puts
      // the drift back to a single rounding.
      return st;
    }
    return collect(cg_tol_, cg_log_rows_, cg_log_, res, s);
  }

  // per-load CG state, all_done and the residual log of a new solve
  int init_state(double tol, int maxiter, int log_cap, cudaStream_t s) {
    const int LK = g_.L * g_.K;
    const bool per_load = (int)load_tol_.size() == LK;
    for (int l = 0; l < LK; ++l) {
      LoadState& h = h_st_[l];
      std::memset(&h, 0, sizeof(LoadState));
      h.tol = per_load ? load_tol_[l] : tol;
      h.maxiter = maxiter;
      h.guard = sizeof(R) == 4 ? 4.0 : 0.0;
    }
    load_tol_.clear();
    FHP_CHECK(cudaMemcpyAsync(st_, h_st_, LK * sizeof(LoadState), cudaMemcpyHostToDevice, s));
    FHP_CHECK(cudaMemsetAsync(all_done_, 0, sizeof(int), s));
    cg_log_rows_ = std::max(1, std::min(log_cap, maxiter + 1));
    cg_log_ = static_cast<double*>(scratch(SCR_LOG, (size_t)cg_log_rows_ * LK * sizeof(double)));
    if (!cg_log_) return ST_OOM;
    FHP_CHECK(cudaMemsetAsync(cg_log_, 0, (size_t)cg_log_rows_ * LK * sizeof(double), s));
    return ST_OK;
  }

  // The iterations of a solve, in chunks between host checks of all_done.
  // One iteration's launches are captured once per solve into a CUDA graph
  // and replayed per iteration (one launch instead of about ten: small grids
  // are launch-bound).  Direct launches when profiling (the per-kernel events)
  // or when the stream cannot be captured (the legacy default stream).
  template <typename F>
  int iterate(int maxiter, cudaStream_t s, F&& one_iteration) {
    int st = ST_OK;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long per_iter = 0;
    if (!prof.on && maxiter > 0 &&
        cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const long long l0 = launches;
      const int cst = one_iteration();
      const cudaError_t e = cudaStreamEndCapture(s, &graph);
      per_iter = launches - l0;
      launches = l0;
      if (cst != ST_OK || e != cudaSuccess || !graph ||
          cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        graph = nullptr;
        gexec = nullptr;
      }
    }
    (void)cudaGetLastError();  // a refused capture leaves no error behind
    auto release_graph = [&]() {
      if (gexec) cudaGraphExecDestroy(gexec);
      if (graph) cudaGraphDestroy(graph);
    };
    int done_iters = 0;
    int chunk = 2;
    while (done_iters < maxiter) {
      FHP_CHECK(cudaMemcpyAsync(h_done_, all_done_, sizeof(int), cudaMemcpyDeviceToHost, s));
      FHP_CHECK(cudaStreamSynchronize(s));
      if (*h_done_) break;
      const int nit = std::min(chunk, maxiter - done_iters);
      for (int it = 0; it < nit; ++it) {
        if (gexec) {
          const cudaError_t e = cudaGraphLaunch(gexec, s);
          if (e != cudaSuccess) {
            set_error(std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
            release_graph();
            return ST_CUDA;
          }
          launches += per_iter;
        } else if ((st = one_iteration()) != ST_OK) {
          release_graph();
          return st;
        }
      }
      done_iters += nit;
      chunk = std::min(chunk * 2, 32);
    }
    release_graph();
    return ST_OK;
  }

  // a kernel's bounded wait ran out since the last check (*h_err_ read after a
  // synchronisation): the error is reported once and the word cleared
  int take_err(cudaStream_t s) {
    if (!*h_err_) return ST_OK;
    *h_err_ = 0;
    cudaMemsetAsync(err_, 0, sizeof(int), s);
    set_error("a tile load of the integration pass did not complete in its wait limit");
    return ST_TIMEOUT;
  }

  // per-load results of a solve (solver.py:137-138) from the device state
  int collect(double tol, int log_rows, const double* dlog, SolveResult& res, cudaStream_t s) {
    const int LK = g_.L * g_.K;   // every cell's loads, cell-major
    FHP_CHECK(cudaMemcpyAsync(h_st_, st_, LK * sizeof(LoadState), cudaMemcpyDeviceToHost, s));
    res.res_log.assign((size_t)log_rows * LK, 0.0);
    FHP_CHECK(cudaMemcpyAsync(res.res_log.data(), dlog, (size_t)log_rows * LK * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaMemcpyAsync(h_err_, err_, sizeof(int), cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaStreamSynchronize(s));
    if (int st = take_err(s)) return st;
    res.kit.resize(LK);
    res.norm_res.resize(LK);
    res.status.resize(LK);
    res.iterations_run = 0;
    for (int l = 0; l < LK; ++l) {
      const LoadState& h = h_st_[l];
      res.kit[l] = h.kit;
      res.norm_res[l] = h.kit == 0 ? 0.0 : h.norm_res;  // solver.py:137-138
      int sl = h.status;
      if (sl == 0 && h.norm_res > tol && h.kit > 0) sl = ST_NONCONVERGED;
      res.status[l] = sl;
      res.iterations_run = std::max(res.iterations_run, h.kit);
    }
    return ST_OK;  // per-load statuses are reported in res.status
  }

  // ---- spectral CG of band plans ---------------------------------------------
  // The iterates x, r, p, Ap are kept as half spectra of the N grid in z form
  // (k_half_weight): the band operator then starts at the pad to the
  // integration grid and ends at the band projection, with no transform on
  // the N grid inside the iteration, and the grid-mean inner products are
  // Euclidean sums over z (fin kernels with a unit mean factor).  CG is the
  // same recursion on the same operator in an orthogonal basis (Parseval), so
  // iterates, residual norms and stopping tests are the reference's up to
  // roundoff.  The initial residual is projected onto range(G).
  void set_spectral_cg(bool on) override { spectral_cg_ = on; }
  void set_integration_kernel(int kind) override { integ_kernel_ = kind; }

  int ensure_spectral() {
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    if (!zb_) FHP_CHECK(cudaMalloc(&zb_, 4 * nz * sizeof(cplx<R>)));
    gz_ = g_;
    gz_.M = 2LL * g_.n0 * g_.n1 * g_.n2h;
    // partial sums of the spectral projection pass: one per CTA (the buffer
    // grows once per plan; cudaFree waits for work that still uses it)
    projf_parts_ = band_axis_ctas(BAND_DOWN_F, spectral_proj_axis(), lb1_.dev, l1_.dev);
    if (projf_parts_ > nparts_max_) {
      double* np = nullptr;
      FHP_CHECK(cudaMalloc(&np, (size_t)projf_parts_ * kMaxLoads * kMaxLoads * sizeof(double)));
      cudaFree(partials_);
      partials_ = np;
      nparts_max_ = (int)projf_parts_;
    }
    return ST_OK;
  }

  // the last band pass of the spectral operator: axis 1 (3D) or the line axis (2D)
  BandAxis spectral_proj_axis() const {
    const long long n2h = g_.n2h;
    if (g_.dim == 3) return BandAxis{gi_.n1, g_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, g_.n0, g_.n0, 1, 0, 0};
    return BandAxis{gi_.n1, g_.n1, g_.n1, gi_.n1, gp_.h[0], n2h, 1, 1, 0, 0, 0};
  }

  // field (plan precision, real) -> z form of its half spectrum
  int to_z(const R* field, cplx<R>* z, cudaStream_t s) {
    int st = forward_spectrum(field, S_, s);
    if (st != ST_OK) return st;
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    k_half_weight<R><<<grid_for(nz), kThreads, 0, s>>>(S_, z, (long long)nz, g_.n2h, g_.n2,
                                                       1.0 / (double)g_.M, 1);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // z form -> real field
  int from_z(const cplx<R>* z, R* field, cudaStream_t s) {
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    k_half_weight<R><<<grid_for(nz), kThreads, 0, s>>>(z, S_, (long long)nz, g_.n2h, g_.n2, 1.0,
                                                       0);
    FHP_LAUNCHED();
    return inverse_spectrum(S_, field, 1.0, s);
  }

  // z <- G z (orthogonal projection onto range(G), unit scale)
  int spec_green(cplx<R>* z, cudaStream_t s) {
    GreenParams gpo = gp_;
    gpo.scale = 1.0;
    const size_t nf = (size_t)g_.L * g_.n0 * g_.n1 * g_.n2h;
    if (gp_.physics == 0) k_spec_green<R, 0><<<grid_for(nf), kThreads, 0, s>>>(z, g_, gpo);
    else k_spec_green<R, 1><<<grid_for(nf), kThreads, 0, s>>>(z, g_, gpo);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // zap = A p in z form on the band (without G: the update projects it),
  // p = r + beta p first (all in the spectral buffers), partial <p, Ap> per
  // CTA of the last pass
  int spectral_operator(const cplx<R>* zr, cplx<R>* zp, cplx<R>* zap, cudaStream_t s) {
    int st;
    const long long n2h = g_.n2h;
    cplx<R>* SA = S_;
    cplx<R>* SB = SB_;
    cplx<R>* Sbig;
    if (g_.dim == 3) {
      BandAxis a0{g_.n0, gi_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)g_.n1 * n2h, 1, 1, 2,
                  (int)n2h, g_.n1};
      if ((st = band_axis(BAND_PAD_PUPD, zr, SB, a0, lb0_.dev, lb0_.dev, true, s,
                          "band_pad_pupd_axis0", zp)) != ST_OK) return st;
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, gi_.n0, g_.n0, 1, 0, 0};
      if ((st = band_axis(BAND_PAD, SB, SA, a1, lb1_.dev, lb1_.dev, true, s,
                          "band_pad_axis1")) != ST_OK) return st;
      Sbig = SA;
    } else {
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[0], n2h, 1, 1, 0, 0, 0};
      if ((st = band_axis(BAND_PAD_PUPD, zr, SB, a1, lb1_.dev, lb1_.dev, true, s,
                          "band_pad_pupd_axis0", zp)) != ST_OK) return st;
      Sbig = SB;
    }
    // the z-form input carries 1 / prod(N) already: unit coefficient scale
    if ((st = band_last_pass(coef_kind_, Sbig, (R)1, true, s)) != ST_OK) return st;
    if (g_.dim == 3) {
      BandAxis a0{gi_.n0, g_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)gi_.n1 * n2h, 1, 1, 2, 0, 0};
      if ((st = band_axis(BAND_DOWN, SA, SB, a0, lb0_.dev, l0_.dev, true, s,
                          "band_down_axis0")) != ST_OK) return st;
    }
    return band_axis(BAND_DOWN_F, SB, zap, spectral_proj_axis(), lb1_.dev, l1_.dev, true, s,
                     "band_downf_axis1", zp, partials_);
  }

  // zout = A u on the band in z form, times gp_.scale, from the plain
  // normalised half spectra of u in S_ (N layout, consumed): the passes of
  // spectral_operator without the direction update, every load
  int spectral_apply_plain(cplx<R>* zout, cudaStream_t s) {
    int st;
    const long long n2h = g_.n2h;
    cplx<R>* Sbig;
    if (g_.dim == 3) {
      BandAxis a0{g_.n0, gi_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)g_.n1 * n2h, 1, 1, 2,
                  (int)n2h, g_.n1};
      if ((st = band_axis(BAND_PAD, S_, SB_, a0, lb0_.dev, lb0_.dev, false, s,
                          "band_pad_axis0")) != ST_OK) return st;
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, gi_.n0, g_.n0, 1, 0, 0};
      if ((st = band_axis(BAND_PAD, SB_, S_, a1, lb1_.dev, lb1_.dev, false, s,
                          "band_pad_axis1")) != ST_OK) return st;
      Sbig = S_;
    } else {
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[0], n2h, 1, 1, 0, 0, 0};
      if ((st = band_axis(BAND_PAD, S_, SB_, a1, lb1_.dev, lb1_.dev, false, s,
                          "band_pad_axis0")) != ST_OK) return st;
      Sbig = SB_;
    }
    if ((st = band_last_pass(coef_kind_, Sbig, (R)1, false, s)) != ST_OK) return st;
    if (g_.dim == 3) {
      BandAxis a0{gi_.n0, g_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)gi_.n1 * n2h, 1, 1, 2, 0, 0};
      if ((st = band_axis(BAND_DOWN, S_, SB_, a0, lb0_.dev, l0_.dev, false, s,
                          "band_down_axis0")) != ST_OK) return st;
    }
    return band_axis(BAND_DOWN_F, SB_, zout, spectral_proj_axis(), lb1_.dev, l1_.dev, false, s,
                     "band_downf_axis1");
  }

  // B = G A (-E) of every load (applications.py:58 Afun(-E)) through the
  // spectral passes: the constant field -E has the single frequency 0, so the
  // solve-grid transforms of the real-field operator reduce to a zeroed
  // spectrum and one write; G in z form, then the real field.
  int spectral_rhs(int proj, R* b, cudaStream_t s) {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    int st = ensure_spectral();
    if (st != ST_OK) return st;
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    cplx<R>* zo = zb_ + 3 * nz;
    if ((st = spectral_rhs_z(proj, zo, s)) != ST_OK) return st;
    return from_z(zo, b, s);
  }

  // G A (-E) in z form into zo (not one of the pass buffers S_, SB_)
  int spectral_rhs_z(int proj, cplx<R>* zo, cudaStream_t s) {
    const long long nzc = (long long)g_.n0 * g_.n1 * g_.n2h;
    const size_t nz = (size_t)g_.L * g_.dv * nzc;
    FHP_CHECK(cudaMemsetAsync(S_, 0, nz * sizeof(cplx<R>), s));
    k_z_macro<R><<<1, 32, 0, s>>>(S_, nzc, g_.L, g_.dv, -1.0);
    FHP_LAUNCHED();
    gp_.proj = proj;
    // s A (-E) on the band (the operator scale s / prod(B)), then G (unit scale)
    int st = spectral_apply_plain(zo, s);
    if (st != ST_OK) return st;
    return spec_green(zo, s);
  }

  // A_H[i][j] = <A u_i, u_j> (postprocess.py:53-70) through the spectral
  // passes: u in z form (+ E at frequency 0), A u on the band in z form with
  // the unscaled coefficient (1 / prod(B)), then the Euclidean sums over the
  // z entries, which are grid means (Parseval)
  int spectral_energy(const R* X, int add_macro, double* AH, cudaStream_t s) {
    int st = ensure_spectral();
    if (st != ST_OK) return st;
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    cplx<R>* zu = zb_ + 2 * nz;
    if ((st = to_z(X, zu, s)) != ST_OK) return st;
    return spectral_energy_z(zu, add_macro, AH, s);
  }

  // the same from the z form of X in zu (a spectral buffer other than the
  // last, which takes A u; E is added in place)
  int spectral_energy_z(cplx<R>* zu, int add_macro, double* AH, cudaStream_t s) {
    const long long nzc = (long long)g_.n0 * g_.n1 * g_.n2h;
    const size_t nz = (size_t)g_.L * g_.dv * nzc;
    cplx<R>* zw = zb_ + 3 * nz;
    if (add_macro) {
      k_z_macro<R><<<1, 32, 0, s>>>(zu, nzc, g_.L, g_.dv, 1.0);
      FHP_LAUNCHED();
    }
    k_half_weight<R><<<grid_for(nz), kThreads, 0, s>>>(zu, S_, (long long)nz, g_.n2h, g_.n2, 1.0,
                                                       0);
    FHP_LAUNCHED();
    const int proj_saved = gp_.proj;
    const double scale_saved = gp_.scale;
    gp_.proj = 0;
    gp_.scale = 1.0 / (double)gi_.M;
    int st = spectral_apply_plain(zw, s);
    gp_.proj = proj_saved;
    gp_.scale = scale_saved;
    if (st != ST_OK) return st;
    if ((st = cross_dot(reinterpret_cast<const R*>(zw), reinterpret_cast<const R*>(zu), gz_, 0,
                        (double)gz_.M * sizeof(R), s)) != ST_OK) return st;
    return finish_energy(1.0, AH, s);
  }

  // per-CTA partial sums of W_i . (X_j (+ E_j)) over g.M values per component
  int cross_dot(const R* W, const R* X, const GridDims& g, int add_macro, double comp_bytes,
                cudaStream_t s) {
    const int pk = pbeg("band_cross_dot", 2.0 * g.L * g.dv * comp_bytes, s);
    switch (g.L) {
      case 1: k_cross_dot<R, 1><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
      case 2: k_cross_dot<R, 2><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
      case 3: k_cross_dot<R, 3><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
      case 4: k_cross_dot<R, 4><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
      case 5: k_cross_dot<R, 5><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
      default: k_cross_dot<R, 6><<<red_ctas_, 256, 0, s>>>(W, X, partials_, g, add_macro); break;
    }
    pend(pk, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // A_H = factor x the sum of the cross-dot partials, to the host
  int finish_energy(double factor, double* AH, cudaStream_t s) {
    k_sum_partials<<<1, kThreads, 0, s>>>(partials_, red_ctas_, g_.L * g_.L, factor, ad_);
    FHP_LAUNCHED();
    FHP_CHECK(cudaMemcpyAsync(AH, ad_, (size_t)g_.L * g_.L * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaMemcpyAsync(h_err_, err_, sizeof(int), cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaStreamSynchronize(s));
    return take_err(s);
  }

  int spectral_iteration(cplx<R>* zx, cplx<R>* zr, cplx<R>* zp, cplx<R>* zap, double* dlog,
                         int log_rows, cudaStream_t s) {
    int st = spectral_operator(zr, zp, zap, s);
    if (st != ST_OK) return st;
    k_fin_pap<<<g_.L, kThreads, 0, s>>>(partials_, (int)projf_parts_, st_, g_.L, 1.0, all_done_);
    FHP_LAUNCHED();
    const int C = g_.L * g_.dv;
    // x += alpha p, r -= alpha G(Ap): the operator's projection happens here
    const int ux = std::max(1, red_ctas_ / g_.L);
    const int pk = pbeg("cg_update_spectral", 6.0 * (double)C * gz_.M * sizeof(R), s);
    GreenParams gpo = gp_;
    gpo.scale = 1.0;
    const FastDiv dn1 = make_fastdiv((unsigned)g_.n1);
    const dim3 ug((unsigned)ux, (unsigned)g_.L);
    if (gp_.physics == 0)
      k_cg_update_spec<R, 0><<<ug, kThreads, 0, s>>>(zx, zr, zp, zap, partials_, g_, gpo, dn1,
                                                     st_, all_done_);
    else
      k_cg_update_spec<R, 1><<<ug, kThreads, 0, s>>>(zx, zr, zp, zap, partials_, g_, gpo, dn1,
                                                     st_, all_done_);
    pend(pk, s);
    FHP_LAUNCHED();
    k_fin_rr<<<g_.L, kThreads, 0, s>>>(partials_, ux * g_.L, st_, g_.L, 1.0, dlog, log_rows,
                                       all_done_);
    FHP_LAUNCHED();
    k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int spectral_cg_begin(int proj, const R* b, const R* x0, double tol, int maxiter,
                        int log_cap, cudaStream_t s) {
    int st = ensure_spectral();
    if (st != ST_OK) return st;
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    cplx<R>* zx = zb_;
    cplx<R>* zr = zb_ + nz;
    cplx<R>* zp = zb_ + 2 * nz;
    // x = x0 ; R = B - A x0 (solver.py:114-117), then both in z form, R
    // projected onto range(G)
    const R* rsrc = b;
    if (x0) {
      if ((st = ensure_cg_buffers()) != ST_OK) return st;
      if ((st = apply_ex(proj, x0, ap_, s, true)) != ST_OK) return st;
      FHP_CHECK(cudaMemcpyAsync(r_, b, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
      k_axpby<R><<<grid_for(n), kThreads, 0, s>>>((long long)n, -1.0, ap_, 1.0, r_);
      FHP_LAUNCHED();
      rsrc = r_;
      if ((st = to_z(x0, zx, s)) != ST_OK) return st;
      if ((st = spec_green(zx, s)) != ST_OK) return st;
    } else {
      FHP_CHECK(cudaMemsetAsync(zx, 0, nz * sizeof(cplx<R>), s));
    }
    if ((st = to_z(rsrc, zr, s)) != ST_OK) return st;
    return spectral_cg_start(tol, maxiter, log_cap, s);
  }

  // the rest of the spectral CG set-up, x and r (z form) in place: r
  // projected onto range(G), p = r, the per-load state and <r, r>
  int spectral_cg_start(double tol, int maxiter, int log_cap, cudaStream_t s) {
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    cplx<R>* zr = zb_ + nz;
    cplx<R>* zp = zb_ + 2 * nz;
    int st = spec_green(zr, s);
    if (st != ST_OK) return st;
    FHP_CHECK(cudaMemcpyAsync(zp, zr, nz * sizeof(cplx<R>), cudaMemcpyDeviceToDevice, s));
    if ((st = init_state(tol, maxiter, log_cap, s)) != ST_OK) return st;
    k_dot<R><<<red_ctas_, kThreads, 0, s>>>(reinterpret_cast<const R*>(zr),
                                            reinterpret_cast<const R*>(zr), partials_, gz_);
    FHP_LAUNCHED();
    k_fin_init<<<1, 32, 0, s>>>(partials_, red_ctas_, st_, g_.L, 1.0, cg_log_, cg_log_rows_);
    FHP_LAUNCHED();
    k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L, all_done_);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // rhs_macro, CG from x = 0 and the energy with every vector kept in z form:
  // the right-hand side goes straight into r, the solution's z form into the
  // energy, and the real solution field is made only when asked for
  int homogenize(int proj, double tol, int maxiter, void* bv, void* xv, bool keep_x, double* AH,
                 SolveResult& res, cudaStream_t s) override {
    if (!(band_ && spectral_cg_))
      return EngineBase::homogenize(proj, tol, maxiter, bv, xv, keep_x, AH, res, s);
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    int st = ensure_spectral();
    if (st != ST_OK) return st;
    const size_t nz = (size_t)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h;
    cplx<R>* zx = zb_;
    cplx<R>* zr = zb_ + nz;
    gp_.proj = proj;
    cg_spectral_ = true;
    cg_proj_ = proj;
    cg_tol_ = tol;
    cg_x_ = static_cast<R*>(xv);
    FHP_CHECK(cudaMemsetAsync(zx, 0, nz * sizeof(cplx<R>), s));
    if ((st = spectral_rhs_z(proj, zr, s)) != ST_OK) return st;   // r = b - A 0
    if ((st = spectral_cg_start(tol, maxiter, 1, s)) != ST_OK) return st;
    if ((st = iterate(maxiter, s, [&]() { return cg_step(s); })) != ST_OK) return st;
    // as cg_end: FP32 iterates projected once more
    if (sizeof(R) == 4 && (st = spec_green(zx, s)) != ST_OK) return st;
    if (keep_x && (st = from_z(zx, cg_x_, s)) != ST_OK) return st;
    if ((st = collect(tol, cg_log_rows_, cg_log_, res, s)) != ST_OK) return st;
    return spectral_energy_z(zx, 1, AH, s);   // x is not needed after this
  }

  // A_H[i][j] = <A u_i, u_j>, u_i = X_i (+ E_i)  (postprocess.py:53-70)
  int energy(const void* Xv, int add_macro, double* AH, cudaStream_t s) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    const R* X = static_cast<const R*>(Xv);
    const int L = g_.L;
    if (band_) return spectral_cg_ ? spectral_energy(X, add_macro, AH, s)
                                   : band_energy(X, add_macro, AH, s);
    switch (coef_kind_) {
      case COEF_ISO: k_energy<R, COEF_ISO><<<dim3(red_ctas_, g_.K), 128, 0, s>>>(X, A_, partials_, g_, add_macro); break;
      case COEF_SYM: k_energy<R, COEF_SYM><<<dim3(red_ctas_, g_.K), 128, 0, s>>>(X, A_, partials_, g_, add_macro); break;
      default: k_energy<R, COEF_FULL><<<dim3(red_ctas_, g_.K), 128, 0, s>>>(X, A_, partials_, g_, add_macro); break;
    }
    FHP_LAUNCHED();
    k_sum_partials<<<g_.K, kThreads, 0, s>>>(partials_, red_ctas_, L * L, 1.0 / (double)g_.M, ad_);
    FHP_LAUNCHED();
    FHP_CHECK(cudaMemcpyAsync(AH, ad_, (size_t)g_.K * L * L * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaStreamSynchronize(s));
    return ST_OK;
  }

  int energy_gradient(const void* Xv, int add_macro, const double* W, double* grad,
                      cudaStream_t s) override {
    if (!A_) { set_error("coefficient not set"); return ST_BAD_ARG; }
    if (band_) {
      set_error("coefficient gradient needs the coefficient on the solve grid "
                "(GaNi or full-grid plan), not on a band integration grid");
      return ST_BAD_ARG;
    }
    LoadMat lm{};
    for (int i = 0; i < g_.L * g_.L; ++i) lm.w[i] = W[i];
    const R* X = static_cast<const R*>(Xv);
    const double invM = 1.0 / (double)g_.M;
    switch (coef_kind_) {
      case COEF_ISO:
        k_energy_grad<R, COEF_ISO><<<red_ctas_, 128, 0, s>>>(X, grad, g_, add_macro, lm, invM);
        break;
      case COEF_SYM:
        k_energy_grad<R, COEF_SYM><<<red_ctas_, 128, 0, s>>>(X, grad, g_, add_macro, lm, invM);
        break;
      default:
        k_energy_grad<R, COEF_FULL><<<red_ctas_, 128, 0, s>>>(X, grad, g_, add_macro, lm, invM);
        break;
    }
    FHP_LAUNCHED();
    return ST_OK;
  }

  int forward_spectrum(const void* xv, void* spec, cudaStream_t s) override {
    cplx<R>* Sp = static_cast<cplx<R>*>(spec);
    int st = fwd_passes(COEF_NONE, false, static_cast<const R*>(xv), nullptr, nullptr, Sp,
                        false, s);
    if (st != ST_OK) return st;
    // complete the forward transform on the first real axis
    const int d = g_.dim;
    const LineDev<R>& lf = d == 3 ? l0_.dev : l1_.dev;
    const long long inner = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    const int T = d == 3 ? T0_ : tile_cols(lf.ld, 1, inner);
    dim3 grid((unsigned)((inner + T - 1) / T), (unsigned)(g_.L * g_.dv), (unsigned)g_.K);
    k_c2c_axis<R, false><<<grid, kThreads, (size_t)T * lf.ld * sizeof(cplx<R>), s>>>(
        Sp, d == 3 ? g_.n0 : g_.n1, inner, lf, T, nullptr, nullptr, 0, g_.ss, g_.L);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int inverse_spectrum(void* spec, void* xv, double scale, cudaStream_t s) override {
    cplx<R>* Sp = static_cast<cplx<R>*>(spec);
    const int d = g_.dim;
    const LineDev<R>& lf = d == 3 ? l0_.dev : l1_.dev;
    const long long inner = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    const int T = d == 3 ? T0_ : tile_cols(lf.ld, 1, inner);
    dim3 grid((unsigned)((inner + T - 1) / T), (unsigned)(g_.L * g_.dv), (unsigned)g_.K);
    k_c2c_axis<R, true><<<grid, kThreads, (size_t)T * lf.ld * sizeof(cplx<R>), s>>>(
        Sp, d == 3 ? g_.n0 : g_.n1, inner, lf, T, nullptr, nullptr, 0, g_.ss, g_.L);
    FHP_LAUNCHED();
    return inv_passes(Sp, static_cast<R*>(xv), (R)scale, false, nullptr, false, s);
  }

  int residual(const void* b, const void* ax, void* r, double* sumsq,
               cudaStream_t s) override {
    k_residual<R><<<dim3(red_ctas_, g_.K), kThreads, 0, s>>>(static_cast<const R*>(b),
                                                 static_cast<const R*>(ax), static_cast<R*>(r),
                                                 partials_, g_);
    FHP_LAUNCHED();
    k_sum_partials<<<g_.K, kThreads, 0, s>>>(partials_, red_ctas_, g_.L, 1.0, ad_);
    FHP_LAUNCHED();
    FHP_CHECK(cudaMemcpyAsync(sumsq, ad_, (size_t)g_.K * g_.L * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    FHP_CHECK(cudaStreamSynchronize(s));
    return ST_OK;
  }

  // scale[] holds one value per load of every cell (host); the values go to
  // the plan's device scale slots (the copy from pageable memory has read
  // them when it returns)
  int scale_from64(const double* src, const double* scale, void* dst, cudaStream_t s) override {
    const size_t LK = (size_t)g_.L * g_.K;
    FHP_CHECK(cudaMemcpyAsync(dscale_, scale, LK * sizeof(double), cudaMemcpyHostToDevice, s));
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    k_scale_from64<R><<<grid_for(n), kThreads, 0, s>>>(src, static_cast<R*>(dst), (long long)n,
                                                        (long long)g_.dv * g_.M, dscale_);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int add_scaled_to64(const void* d, const double* scale, double* x, cudaStream_t s) override {
    const size_t LK = (size_t)g_.L * g_.K;
    double* ds = dscale_ + (size_t)g_.K * kMaxLoads;
    FHP_CHECK(cudaMemcpyAsync(ds, scale, LK * sizeof(double), cudaMemcpyHostToDevice, s));
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    k_add_scaled_to64<R><<<grid_for(n), kThreads, 0, s>>>(static_cast<const R*>(d), x,
                                                           (long long)n, (long long)g_.dv * g_.M,
                                                           ds);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int ga_gather(const void* spec_src, const PlanConfig& src, const int* d_index,
                const double* d_weight, void* spec_dst, cudaStream_t s) override {
    const int d = cfg_.dim;
    const int P0 = d == 3 ? src.N[0] : 1, P1 = src.N[d - 2], P2 = src.N[d - 1];
    k_ga_gather<R><<<grid_for(spec_elems_), kThreads, 0, s>>>(
        static_cast<const cplx<R>*>(spec_src), static_cast<cplx<R>*>(spec_dst), g_.L * g_.dv,
        P0, P1, P2, g_.n0, g_.n1, g_.n2, d_index, d_weight);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int pad_spectrum(const void* spec_src, const PlanConfig& src, void* spec_dst,
                   cudaStream_t s) override {
    const int d = cfg_.dim;
    const int N0 = d == 3 ? src.N[0] : 1, N1 = src.N[d - 2], N2 = src.N[d - 1];
    const size_t tot = spec_elems_;
    k_spectrum_pad<R><<<grid_for(tot), kThreads, 0, s>>>(
        static_cast<const cplx<R>*>(spec_src), static_cast<cplx<R>*>(spec_dst), g_.L * g_.dv, d,
        N0, N1, N2, g_.n0, g_.n1, g_.n2);
    FHP_LAUNCHED();
    return ST_OK;
  }

 private:
  PlanConfig cfg_;
  GridDims g_{};
  GreenParams gp_{};
  DevLine<R> l0_, l1_, l2_;
  cplx<R>* S_ = nullptr;
  size_t spec_elems_ = 0;
  R* A_ = nullptr;
  int coef_kind_ = 0;
  R *r_ = nullptr, *p_ = nullptr, *ap_ = nullptr;
  double* partials_ = nullptr;
  void* scr_[kScratchSlots] = {};
  size_t scr_bytes_[kScratchSlots] = {};
  double* ad_ = nullptr;
  double* dscale_ = nullptr;   // per-load scales of the refinement (2 x cells x loads)
  std::vector<double> load_tol_;   // per-load tolerances of the next solve (set_load_tols)
  LoadState* st_ = nullptr;
  LoadState* h_st_ = nullptr;
  int* all_done_ = nullptr;
  int* h_done_ = nullptr;
  // a bounded wait of a kernel ran out (device word, pinned host copy)
  int* err_ = nullptr;
  int* h_err_ = nullptr;
  int rows_ = 1, row_ctas_ = 1, T1_ = 1, Tp_ = 1, T0_ = 1;
  bool c2r_stage_ = false;   // k_c2r_last stages its input spectra in shared memory
  size_t smem_rows_ = 0;
  int nsm_ = 1, red_ctas_ = 1, nparts_max_ = 1;

  // algorithmic bytes of the passes (each input read once, each output written once)
  double field_bytes() const { return (double)g_.K * g_.L * g_.dv * g_.M * sizeof(R); }
  // the solve grid's half spectrum (the buffer of band plans is larger: it
  // also holds the integration grid's spectra)
  double spec_bytes() const {
    return (double)g_.K * g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h * 2 * sizeof(R);
  }
  double coef_bytes() const {
    const int dv = g_.dv;
    const int c = coef_kind_ == COEF_ISO ? 1 : coef_kind_ == COEF_SYM ? dv * (dv + 1) / 2
                : coef_kind_ == COEF_FULL ? dv * dv : 0;
    return (double)g_.K * c * (band_ ? gi_.M : g_.M) * sizeof(R);
  }
  int pbeg(const char* name, double bytes, cudaStream_t s) {
    if (!prof.on) return -1;
    const std::string tag = std::string(name) + (sizeof(R) == 8 ? "<f64>" : "<f32>");
    const int k = prof.kind_of(tag, bytes);
    prof.begin(k, s);
    return k;
  }
  void pend(int k, cudaStream_t s) {
    if (k >= 0) prof.end(s);
  }

  static unsigned grid_for(size_t n) {
    size_t b = (n + kThreads - 1) / kThreads;
    return (unsigned)std::max<size_t>(1, std::min<size_t>(b, 65535 * 4));
  }

  int tile_cols(int nf, int lines_per_col, long long inner,
                int target = kTargetElems, size_t budget = kSmemBudget) const {
    const size_t per = (size_t)lines_per_col * nf * sizeof(cplx<R>);
    int T = std::max(1, target / (lines_per_col * nf));
    T = std::min(T, 32);
    T = (int)std::min<size_t>(T, std::max<size_t>(1, budget / per));
    T = (int)std::min<long long>(T, inner);
    T = std::max(T, 1);
    while (T & (T - 1)) T &= T - 1;  // kernels index tiles with shifts: a power of two
    return T;
  }

  int make_line(int n, DevLine<R>& out) {
    LinePlanHost h;
    if (!build_line_plan(n, h, p2_two_stage_len<R>())) {
      set_error("cannot plan FFT length " + std::to_string(n));
      return ST_BAD_ARG;
    }
    if (h.nst > kMaxStages) { set_error("too many FFT stages"); return ST_BAD_ARG; }
    const size_t ntw = h.tw.size(), nch = h.chirp.size(), nbh = h.bhat.size();
    const size_t bytes = (ntw + nch + nbh) * sizeof(cplx<R>) + h.pos.size() * sizeof(int) + 64;
    FHP_CHECK(cudaMalloc(&out.mem, bytes));
    std::vector<unsigned char> host(bytes, 0);
    cplx<R>* c = reinterpret_cast<cplx<R>*>(host.data());
    auto put = [&](const std::vector<std::complex<long double>>& v, size_t off) {
      for (size_t i = 0; i < v.size(); ++i) c[off + i] = mkc<R>((R)v[i].real(), (R)v[i].imag());
    };
    put(h.tw, 0);
    put(h.chirp, ntw);
    put(h.bhat, ntw + nch);
    int* ip = reinterpret_cast<int*>(c + ntw + nch + nbh);
    std::memcpy(ip, h.pos.data(), h.pos.size() * sizeof(int));
    FHP_CHECK(cudaMemcpy(out.mem, host.data(), bytes, cudaMemcpyHostToDevice));
    // From pageable memory cudaMemcpy returns once the data is staged, and the
    // DMA runs on the legacy default stream, which does not order work on
    // non-blocking streams: a plan created in a worker thread could start its
    // first solve on such a stream before its tables land.  Wait for it here.
    FHP_CHECK(cudaStreamSynchronize(cudaStreamLegacy));
    cplx<R>* dc = reinterpret_cast<cplx<R>*>(out.mem);
    LineDev<R>& L = out.dev;
    L.n = h.n;
    L.nf = h.nf;
    L.ld = padded_ld(h.nf);
    L.blue = h.blue;
    L.nst = h.nst;
    // compile-time power-of-two stages when the plan's radices are theirs
    L.lg2 = 0;
    {
      int P = 0;
      while ((1 << P) < h.nf) ++P;
      const int K = p2_k_for<R>(P);
      if ((1 << P) == h.nf && P >= kP2Min && P <= kP2Max && h.nst == p2_nst(P, K)) {
        bool same = true;
        for (int s = 0; s < h.nst; ++s) same = same && h.rad[s] == (1 << p2_e(P, s, K));
        if (same) L.lg2 = P;
      }
      // radix 32 exists only in the compile-time two-stage core
      for (int s = 0; s < h.nst; ++s)
        if (h.rad[s] > 17 && L.lg2 == 0) {
          set_error("FFT length " + std::to_string(n) + ": radix without a core");
          return ST_BAD_ARG;
        }
    }
    // compile-time mixed-radix core (its radix order is factor_radices')
    L.mixed = (!h.blue && h.nf == 255 && h.nst == 3 && h.rad[0] == 3 && h.rad[1] == 5 &&
               h.rad[2] == 17) ? 255 : 0;
    int ns = h.nf;
    for (int i = 0; i < kMaxStages; ++i) {
      L.rad[i] = i < h.nst ? h.rad[i] : 1;
      L.dnbl[i] = make_fastdiv((unsigned)(h.nf / L.rad[i]));
      L.dms[i] = make_fastdiv((unsigned)std::max(1, ns / L.rad[i]));
      if (i < h.nst) ns /= h.rad[i];
    }
    L.dn = make_fastdiv((unsigned)h.n);
    L.dnf = make_fastdiv((unsigned)h.nf);
    L.tw = dc;
    L.chirp = nch ? dc + ntw : nullptr;
    L.bhat = nbh ? dc + ntw + nch : nullptr;
    L.pos = reinterpret_cast<const int*>(dc + ntw + nch + nbh);
    return ST_OK;
  }

  int set_attrs() {
    int st = ST_OK;
#define FHP_ATTR(k) if ((st = set_smem_attr(k)) != ST_OK) return st
    FHP_ATTR((k_r2c_last<R, COEF_NONE, false>));
    FHP_ATTR((k_r2c_last<R, COEF_ISO, false>));
    FHP_ATTR((k_r2c_last<R, COEF_SYM, false>));
    FHP_ATTR((k_r2c_last<R, COEF_FULL, false>));
    FHP_ATTR((k_r2c_last<R, COEF_ISO, true>));
    FHP_ATTR((k_r2c_last<R, COEF_SYM, true>));
    FHP_ATTR((k_r2c_last<R, COEF_FULL, true>));
    FHP_ATTR((k_c2c_axis<R, false>));
    FHP_ATTR((k_c2c_axis<R, true>));
    FHP_ATTR((k_proj_first<R, 0>));
    FHP_ATTR((k_proj_first<R, 1>));
    FHP_ATTR((k_c2r_last<R, false>));
    FHP_ATTR((k_c2r_last<R, true>));
    FHP_ATTR((k_r2c_last<R, COEF_NONE, true>));
    FHP_ATTR((k_band_axis<R, BAND_UP, 0>));
    FHP_ATTR((k_band_axis<R, BAND_DOWN, 0>));
    FHP_ATTR((k_band_axis<R, BAND_DOWN_PROJ, 0>));
    FHP_ATTR((k_band_axis<R, BAND_UP_PROJ, 0>));
    FHP_ATTR((k_band_axis<R, BAND_DOWN_PROJ, 1>));
    FHP_ATTR((k_band_axis<R, BAND_UP_PROJ, 1>));
    FHP_ATTR((k_band_axis<R, BAND_PAD, 0>));
    FHP_ATTR((k_band_axis<R, BAND_PAD_PUPD, 0>));
    FHP_ATTR((k_band_axis<R, BAND_DOWN_F, 0>));
    FHP_ATTR((k_band_last<R, COEF_ISO>));
    FHP_ATTR((k_band_last<R, COEF_SYM>));
    FHP_ATTR((k_band_last<R, COEF_FULL>));
    if constexpr (sizeof(R) == 4) {
      FHP_ATTR((k_band_last_r512<R, false>));
      FHP_ATTR((k_band_last_r512<R, true>));
    }
#define FHP_ATTR_P2(P)                              \
    FHP_ATTR((k_band_last_p2<R, COEF_ISO, P>));     \
    FHP_ATTR((k_band_last_p2<R, COEF_SYM, P>));     \
    FHP_ATTR((k_band_last_p2<R, COEF_FULL, P>))
    static_assert(kP2Min == 5 && kP2Max == 10, "k_band_last_p2 instances 2^5 .. 2^10");
    FHP_ATTR_P2(5); FHP_ATTR_P2(6); FHP_ATTR_P2(7); FHP_ATTR_P2(8); FHP_ATTR_P2(9); FHP_ATTR_P2(10);
#undef FHP_ATTR_P2
#undef FHP_ATTR
    return ST_OK;
  }

  int ensure_cg_buffers() {
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M * sizeof(R);
    if (!r_) FHP_CHECK(cudaMalloc(&r_, n));
    if (!p_) FHP_CHECK(cudaMalloc(&p_, n));
    if (!ap_) FHP_CHECK(cudaMalloc(&ap_, n));
    return ST_OK;
  }

  void* scratch(int slot, size_t bytes) override {
    if (slot < 0 || slot >= kScratchSlots) return nullptr;
    if (scr_bytes_[slot] < bytes) {
      // growing frees the old buffer: cudaFree waits for work that still uses it
      if (scr_[slot]) cudaFree(scr_[slot]);
      scr_[slot] = nullptr;
      scr_bytes_[slot] = 0;
      if (cudaMalloc(&scr_[slot], bytes) != cudaSuccess) {
        scr_[slot] = nullptr;
        set_error("out of device memory for plan scratch");
        return nullptr;
      }
      scr_bytes_[slot] = bytes;
    }
    return scr_[slot];
  }

  void release() {
    for (int i = 0; i < kScratchSlots; ++i)
      if (scr_[i]) { cudaFree(scr_[i]); scr_[i] = nullptr; scr_bytes_[i] = 0; }
    for (DevLine<R>* l : {&l0_, &l1_, &l2_, &lb0_, &lb1_, &lb2_})
      if (l->mem) { cudaFree(l->mem); l->mem = nullptr; }
    if (SB_) { cudaFree(SB_); SB_ = nullptr; }
    if (S_) cudaFree(S_);
    if (A_) cudaFree(A_);
    if (r_) cudaFree(r_);
    if (p_) cudaFree(p_);
    if (ap_) cudaFree(ap_);
    if (partials_) cudaFree(partials_);
    if (ad_) cudaFree(ad_);
    if (dscale_) cudaFree(dscale_);
    if (st_) cudaFree(st_);
    if (all_done_) cudaFree(all_done_);
    if (pe_) cudaFree(pe_);
    if (zx_) cudaFree(zx_);
    if (zb_) cudaFree(zb_);
    zb_ = nullptr;
    pe_ = nullptr;
    zx_ = nullptr;
    if (h_done_) cudaFreeHost(h_done_);
    if (h_st_) cudaFreeHost(h_st_);
    if (err_) cudaFree(err_);
    if (h_err_) cudaFreeHost(h_err_);
    err_ = h_err_ = nullptr;
    S_ = nullptr; A_ = nullptr; r_ = p_ = ap_ = nullptr;
    ad_ = dscale_ = nullptr;
  }

  // pass 1 (+ axis-1 forward for 3D); leaves the spectrum ready for the
  // first-axis pass
  int fwd_passes(int coef, bool pupd, const R* x, R* pio, const R* rvec, cplx<R>* Sp,
                 bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const LoadState* st = cg ? st_ : nullptr;
    const dim3 grid1(row_ctas_, g_.K);
    const double b1 = (pupd ? 3.0 : 1.0) * field_bytes() + (coef ? coef_bytes() : 0.0) +
                      spec_bytes();
    const int pk1 = pbeg(pupd ? "r2c_coef_pupd" : (coef ? "r2c_coef" : "r2c"), b1, s);
#define FHP_R2C(C, P)                                                                     \
  k_r2c_last<R, C, P><<<grid1, kThreads, smem_rows_, s>>>(x, pio, rvec, A_, Sp, g_, l2_.dev, \
                                                            rows_, st_, ad)
    if (pupd) {
      switch (coef) {
        case COEF_ISO: FHP_R2C(COEF_ISO, true); break;
        case COEF_SYM: FHP_R2C(COEF_SYM, true); break;
        default: FHP_R2C(COEF_FULL, true); break;
      }
    } else {
      switch (coef) {
        case COEF_NONE: FHP_R2C(COEF_NONE, false); break;
        case COEF_ISO: FHP_R2C(COEF_ISO, false); break;
        case COEF_SYM: FHP_R2C(COEF_SYM, false); break;
        default: FHP_R2C(COEF_FULL, false); break;
      }
    }
#undef FHP_R2C
    pend(pk1, s);
    FHP_LAUNCHED();
    if (g_.dim == 3) {
      dim3 grid((unsigned)((g_.n2h + T1_ - 1) / T1_), (unsigned)(g_.L * g_.dv * g_.n0),
                (unsigned)g_.K);
      const int pk = pbeg("c2c_axis1_fwd", 2.0 * spec_bytes(), s);
      k_c2c_axis<R, false><<<grid, kThreads, (size_t)T1_ * l1_.dev.ld * sizeof(cplx<R>), s>>>(
          Sp, g_.n1, (long long)g_.n2h, l1_.dev, T1_, ad, st, g_.dv * g_.n0, g_.ss, g_.L);
      pend(pk, s);
      FHP_LAUNCHED();
    }
    return ST_OK;
  }

  // axis-1 inverse (3D) + c2r last axis with scale and optional dot
  int inv_passes(cplx<R>* Sp, R* y, R scale, bool dot, const R* pdot, bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const LoadState* st = cg ? st_ : nullptr;
    if (g_.dim == 3) {
      dim3 grid((unsigned)((g_.n2h + T1_ - 1) / T1_), (unsigned)(g_.L * g_.dv * g_.n0),
                (unsigned)g_.K);
      const int pk = pbeg("c2c_axis1_inv", 2.0 * spec_bytes(), s);
      k_c2c_axis<R, true><<<grid, kThreads, (size_t)T1_ * l1_.dev.ld * sizeof(cplx<R>), s>>>(
          Sp, g_.n1, (long long)g_.n2h, l1_.dev, T1_, ad, st, g_.dv * g_.n0, g_.ss, g_.L);
      pend(pk, s);
      FHP_LAUNCHED();
    }
    const dim3 grid1(row_ctas_, g_.K);
    const int pk2 = pbeg(dot ? "c2r_dot" : "c2r", spec_bytes() + (dot ? 2.0 : 1.0) * field_bytes(), s);
    if (dot)
      k_c2r_last<R, true><<<grid1, kThreads, smem_rows_, s>>>(Sp, y, pdot, partials_, g_, l2_.dev,
                                                              rows_, scale, ad, (int)c2r_stage_,
                                                              st);
    else
      k_c2r_last<R, false><<<grid1, kThreads, smem_rows_, s>>>(Sp, y, nullptr, nullptr, g_,
                                                               l2_.dev, rows_, scale, ad,
                                                               (int)c2r_stage_, st);
    pend(pk2, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  int proj_pass(cplx<R>* Sp, bool cg, cudaStream_t s) {
    const int d = g_.dim;
    const LineDev<R>& lp = d == 3 ? l0_.dev : l1_.dev;
    const long long inner = d == 3 ? (long long)g_.n1 * g_.n2h : (long long)g_.n2h;
    dim3 grid((unsigned)((inner + Tp_ - 1) / Tp_), (unsigned)g_.L, (unsigned)g_.K);
    const size_t smem = (size_t)Tp_ * g_.dv * lp.ld * sizeof(cplx<R>);
    const int pk = pbeg("proj_axis0", 2.0 * spec_bytes(), s);
    auto kproj = gp_.physics == 0 ? k_proj_first<R, 0> : k_proj_first<R, 1>;
    kproj<<<grid, kThreads, smem, s>>>(Sp, g_, d == 3 ? g_.n0 : g_.n1, inner, lp, Tp_,
                                                 gp_, cg ? all_done_ : nullptr,
                                                 cg ? st_ : nullptr);
    pend(pk, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // ---- band representation (Ga on the solve grid, A on the integration grid) ----
  // CTAs of a band pass (the partial-sum count of BAND_DOWN_F)
  long long band_axis_ctas(int mode, const BandAxis& ax, const LineDev<R>& L1,
                           const LineDev<R>& L2) const {
    const int T = band_axis_tile(mode, ax, L1, L2);
    const bool projm = mode == BAND_DOWN_PROJ || mode == BAND_UP_PROJ;
    return ((ax.inner + T - 1) / T) * (long long)((projm ? g_.L : g_.L * g_.dv) * ax.mid);
  }

  int band_axis_tile(int mode, const BandAxis& ax, const LineDev<R>& L1,
                     const LineDev<R>& L2) const {
    const bool projm = mode == BAND_DOWN_PROJ || mode == BAND_UP_PROJ;
    const bool padin = mode == BAND_PAD || mode == BAND_PAD_PUPD;
    const int nlc = projm ? g_.dv : 1;
    const int nf = (padin ? 0 : L1.ld) +
                   ((mode == BAND_DOWN || mode == BAND_DOWN_F) ? 0 : L2.ld);
    // twice the usual line target: the axis passes are bound by instruction
    // issue, and more columns per CTA fill the radix stages of every line
    // length (and lengthen the contiguous rows); the register file still
    // allows two CTAs per SM.
    return tile_cols(nf, nlc, ax.inner, 2 * kTargetElems * axis_target_mult_, kSmemBudget);
  }

  int band_axis(int mode, const cplx<R>* in, cplx<R>* out, const BandAxis& ax_in,
                const LineDev<R>& L1, const LineDev<R>& L2, bool cg, cudaStream_t s,
                const char* name, cplx<R>* aux = nullptr, double* parts = nullptr) {
    BandAxis ax = ax_in;
    set_band_divs(ax);
    const bool projm = mode == BAND_DOWN_PROJ || mode == BAND_UP_PROJ;
    const bool padin = mode == BAND_PAD || mode == BAND_PAD_PUPD;
    const int nlc = projm ? g_.dv : 1;
    const int nf = (padin ? 0 : L1.ld) +
                   ((mode == BAND_DOWN || mode == BAND_DOWN_F) ? 0 : L2.ld);
    const int T = band_axis_tile(mode, ax, L1, L2);
    const size_t smem = (size_t)nlc * T * nf * sizeof(cplx<R>);
    if (smem > kSmemMax) { set_error("band line too long for shared memory"); return ST_BAD_ARG; }
    const int outer = projm ? g_.L : g_.L * g_.dv;
    dim3 grid((unsigned)((ax.inner + T - 1) / T), (unsigned)(outer * ax.mid));
    const int* ad = cg ? all_done_ : nullptr;
    const LoadState* st = cg ? st_ : nullptr;
    // algorithmic bytes: each input read once, each output written once; the
    // direction update also reads r and rewrites p, the spectral projection
    // reads p for <p, Ap>
    double bytes = (double)(g_.L * g_.dv) * ax.mid * ax.inner *
                   (ax.n_in + ax.n_out) * sizeof(cplx<R>);
    if (mode == BAND_PAD_PUPD)
      bytes += 2.0 * (g_.L * g_.dv) * ax.mid * ax.inner * ax.n_in * sizeof(cplx<R>);
    if (mode == BAND_DOWN_F && parts)
      bytes += (double)(g_.L * g_.dv) * ax.mid * ax.inner * ax.n_out * sizeof(cplx<R>);
    // the input projection of G A G is the plain orthogonal projection (scale 1);
    // the output projection carries s / prod(B)
    GreenParams gpin = gp_;
    gpin.scale = 1.0;
    const bool scalar = gp_.physics == 0;
    const int pk = pbeg(name, bytes, s);
    switch (mode) {
      case BAND_UP:
        k_band_axis<R, BAND_UP, 0><<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, nullptr, nullptr);
        break;
      case BAND_DOWN:
        k_band_axis<R, BAND_DOWN, 0><<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, nullptr, nullptr);
        break;
      case BAND_UP_PROJ: {
        auto k = scalar ? k_band_axis<R, BAND_UP_PROJ, 0> : k_band_axis<R, BAND_UP_PROJ, 1>;
        k<<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gpin, ad, st, nullptr, nullptr);
        break;
      }
      case BAND_PAD:
        k_band_axis<R, BAND_PAD, 0><<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, nullptr, nullptr);
        break;
      case BAND_PAD_PUPD:
        k_band_axis<R, BAND_PAD_PUPD, 0><<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, aux, nullptr);
        break;
      case BAND_DOWN_F:
        k_band_axis<R, BAND_DOWN_F, 0><<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, aux, parts);
        break;
      default: {
        auto k = scalar ? k_band_axis<R, BAND_DOWN_PROJ, 0> : k_band_axis<R, BAND_DOWN_PROJ, 1>;
        k<<<grid, kThreads, smem, s>>>(in, out, g_, ax, L1, L2, T, gp_, ad, st, nullptr, nullptr);
        break;
      }
    }
    pend(pk, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // last axis on the integration grid: c2r, q = a x cs, r2c, keep the band
  // (in place in Sbig, all loads and comps)
  // the register-resident 512-point integration kernel applies: FP32, an
  // isotropic coefficient, a direct 512-point line, the band within N/4
  bool reg512_applies(int coef) const {
    return sizeof(R) == 4 && coef == COEF_ISO && !lb2_.dev.blue && lb2_.dev.nf == 512 &&
           4 * g_.n2h <= 512 && 2 * g_.n2h - 1 <= g_.n2 + 1;
  }

  int band_last_pass(int coef, cplx<R>* Sbig, R cs, bool cg, cudaStream_t s) {
    const int* ad = cg ? all_done_ : nullptr;
    const long long n2h = g_.n2h;
    if constexpr (sizeof(R) == 4) {
      if (integ_kernel_ >= 1 && reg512_applies(coef)) {
        const long long nrows = (long long)gi_.n0 * gi_.n1;
        const double b4 = 2.0 * (double)(g_.L * g_.dv) * nrows * n2h * sizeof(cplx<R>) +
                          coef_bytes();
        const int pk = pbeg("band_last_coef", b4, s);
        const long long need = (nrows + kR512Warps - 1) / kR512Warps;
        const unsigned ctas =
            (unsigned)std::min<long long>(need, (long long)reg512_ctas_per_sm_ * nsm_);
        // the full band (a 255-point solve line in a 512-point integration
        // line) takes the instantiation without per-frequency tests, and TMA
        // row loads when both maps encode
        const bool full = n2h == 128 && g_.n2 == 255;
        auto kern = full ? k_band_last_r512<R, true> : k_band_last_r512<R, false>;
        CUtensorMap tmS, tmA;
        std::memset(&tmS, 0, sizeof(tmS));
        std::memset(&tmA, 0, sizeof(tmA));
        const int use_tma = (full && integ_kernel_ == 1 &&
                             tmap_rows(&tmS, Sbig, 128, (unsigned long long)g_.L * g_.dv * nrows) &&
                             tmap_rows(&tmA, A_, 256, (unsigned long long)nrows)) ? 1 : 0;
        kern<<<ctas, 32 * kR512Warps, r512_smem_bytes(), s>>>(
            reinterpret_cast<float2*>(Sbig), reinterpret_cast<const float*>(A_), g_, nrows,
            (int)n2h, g_.n2, reinterpret_cast<const float2*>(lb2_.dev.tw), (float)cs, ad, tmS,
            tmA, use_tma, err_, cg ? all_done_ : nullptr);
        pend(pk, s);
        FHP_LAUNCHED();
        return ST_OK;
      }
    }
    const long long nrows = (long long)gi_.n0 * gi_.n1;
    const double b4 = 2.0 * (double)(g_.L * g_.dv) * nrows * n2h * sizeof(cplx<R>) + coef_bytes();
    const int pk = pbeg("band_last_coef", b4, s);
    // rows per CTA: the line target, reduced until lines + staged spectra +
    // staged coefficient fit the per-CTA budget (2 CTAs/SM for FP32)
    const int C = g_.L * g_.dv, np = (C + 1) / 2;
    const int cA = coef == COEF_ISO ? 1 : coef == COEF_SYM ? g_.dv * (g_.dv + 1) / 2 : g_.dv * g_.dv;
    const size_t budget = sizeof(R) == 4 ? kBandLastBudget32 : kBandLastBudget64;
    // staging modes in order of preference: spectra and coefficient, spectra
    // only, none (the lines alone always fit: checked at plan creation)
    int rows = brows_, stage = 3;
    auto smem_of = [&](int r, int stg) {
      return band_last_smem_bytes<R>(r, np, lb2_.dev.ld, C, (int)n2h, cA, gi_.n2, stg);
    };
    for (stage = 3; stage > 0; stage = stage == 3 ? 1 : 0)
      if (smem_of(1, stage) <= budget) break;
    while (rows > 1 && smem_of(rows, stage) > budget) --rows;
    const size_t smem = smem_of(rows, stage);
    if (smem > kSmemMax) { set_error("integration line too long for shared memory"); return ST_BAD_ARG; }
    const unsigned ctas = (unsigned)((nrows + rows - 1) / rows);
    // direct power-of-two integration lines: compile-time stages and phases
    const int lgb = lb2_.dev.blue ? 0 : lb2_.dev.lg2;
#define FHP_BLARGS <<<ctas, kThreads, smem, s>>>(Sbig, A_, g_, nrows, (int)n2h, g_.n2, lb2_.dev, rows, cs, ad, stage)
#define FHP_BL(C)                                                  \
    switch (lgb) {                                               \
      case 5: k_band_last_p2<R, C, 5> FHP_BLARGS; break;          \
      case 6: k_band_last_p2<R, C, 6> FHP_BLARGS; break;          \
      case 7: k_band_last_p2<R, C, 7> FHP_BLARGS; break;          \
      case 8: k_band_last_p2<R, C, 8> FHP_BLARGS; break;          \
      case 9: k_band_last_p2<R, C, 9> FHP_BLARGS; break;          \
      case 10: k_band_last_p2<R, C, 10> FHP_BLARGS; break;        \
      default: k_band_last<R, C> FHP_BLARGS; break;               \
    }
    switch (coef) {
      case COEF_ISO: FHP_BL(COEF_ISO); break;
      case COEF_SYM: FHP_BL(COEF_SYM); break;
      default: FHP_BL(COEF_FULL); break;
    }
#undef FHP_BL
#undef FHP_BLARGS
    pend(pk, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  // inproj: apply G to the input first (G A G): identical on range(G), where
  // the CG iterates live, and annihilates roundoff outside it
  int band_operator(int coef, bool pupd, const R* x, R* pio, const R* rvec, R* y,
                    const R* pdot, cudaStream_t s, bool cg, bool dot, bool inproj = false) {
    int st;
    const int d = g_.dim;
    const int* ad = cg ? all_done_ : nullptr;
    cplx<R>* SA = S_;
    cplx<R>* SB = SB_;
    const long long n2h = g_.n2h;
    // K1: r2c on the solve grid (P update fused)
    {
      const dim3 grid1(row_ctas_);
      const double b1 = (pupd ? 3.0 : 1.0) * field_bytes() + spec_bytes_n();
      const int pk = pbeg(pupd ? "band_r2c_pupd" : "band_r2c", b1, s);
      if (pupd)
        k_r2c_last<R, COEF_NONE, true><<<grid1, kThreads, smem_rows_, s>>>(
            x, pio, rvec, nullptr, SA, g_, l2_.dev, rows_, st_, ad);
      else
        k_r2c_last<R, COEF_NONE, false><<<grid1, kThreads, smem_rows_, s>>>(
            x, pio, rvec, nullptr, SA, g_, l2_.dev, rows_, st_, ad);
      pend(pk, s);
      FHP_LAUNCHED();
    }
    cplx<R>* Sbig;
    if (d == 3 && !inproj) {
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, g_.n0, g_.n0, 1, 0, 0};
      if ((st = band_axis(BAND_UP, SA, SB, a1, l1_.dev, lb1_.dev, cg, s, "band_up_axis1")) != ST_OK) return st;
      BandAxis a0{g_.n0, gi_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)gi_.n1 * n2h, 1, 1, 2, 0, 0};
      if ((st = band_axis(BAND_UP, SB, SA, a0, l0_.dev, lb0_.dev, cg, s, "band_up_axis0")) != ST_OK) return st;
      Sbig = SA;
    } else if (d == 3) {
      // forward DFT_N along axis 1, then axis 0: DFT_N, G, pad, iDFT_B; then pad axis 1
      dim3 grid((unsigned)((n2h + T1_ - 1) / T1_), (unsigned)(g_.L * g_.dv * g_.n0));
      const int pk = pbeg("band_c2c_axis1_fwd", 2.0 * spec_bytes_n(), s);
      k_c2c_axis<R, false><<<grid, kThreads, (size_t)T1_ * l1_.dev.ld * sizeof(cplx<R>), s>>>(
          SA, g_.n1, n2h, l1_.dev, T1_, ad, cg ? st_ : nullptr, g_.dv * g_.n0, g_.ss, g_.L);
      pend(pk, s);
      FHP_LAUNCHED();
      BandAxis a0{g_.n0, gi_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)g_.n1 * n2h, 1, 1, 2,
                  (int)n2h, g_.n1};
      if ((st = band_axis(BAND_UP_PROJ, SA, SB, a0, l0_.dev, lb0_.dev, cg, s, "band_upproj_axis0")) != ST_OK) return st;
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, gi_.n0, g_.n0, 1, 0, 0};
      if ((st = band_axis(BAND_PAD, SB, SA, a1, lb1_.dev, lb1_.dev, cg, s, "band_pad_axis1")) != ST_OK) return st;
      Sbig = SA;
    } else {
      BandAxis a1{g_.n1, gi_.n1, g_.n1, gi_.n1, gp_.h[0], n2h, 1, 1, 0, 0, 0};
      if ((st = band_axis(inproj ? BAND_UP_PROJ : BAND_UP, SA, SB, a1, l1_.dev, lb1_.dev, cg, s,
                          inproj ? "band_upproj_axis0" : "band_up_axis0")) != ST_OK) return st;
      Sbig = SB;
    }
    // K4: last axis on the integration grid with the coefficient
    if ((st = band_last_pass(coef, Sbig, (R)(1.0 / (double)g_.M), cg, s)) != ST_OK) return st;
    if (d == 3) {
      BandAxis a0{gi_.n0, g_.n0, g_.n0, gi_.n0, gp_.h[0], (long long)gi_.n1 * n2h, 1, 1, 2, 0, 0};
      if ((st = band_axis(BAND_DOWN, SA, SB, a0, lb0_.dev, l0_.dev, cg, s, "band_down_axis0")) != ST_OK) return st;
      BandAxis a1{gi_.n1, g_.n1, g_.n1, gi_.n1, gp_.h[1], n2h, g_.n0, g_.n0, 1, 0, 0};
      if ((st = band_axis(BAND_DOWN_PROJ, SB, SA, a1, lb1_.dev, l1_.dev, cg, s, "band_proj_axis1")) != ST_OK) return st;
      // K7: inverse DFT_N along axis 0
      dim3 grid((unsigned)((g_.n1 * n2h + T0_ - 1) / T0_), (unsigned)(g_.L * g_.dv));
      const int pk = pbeg("band_c2c_axis0_inv", 2.0 * spec_bytes_n(), s);
      k_c2c_axis<R, true><<<grid, kThreads, (size_t)T0_ * l0_.dev.ld * sizeof(cplx<R>), s>>>(
          SA, g_.n0, (long long)g_.n1 * n2h, l0_.dev, T0_, ad, cg ? st_ : nullptr, g_.dv, g_.ss, g_.L);
      pend(pk, s);
      FHP_LAUNCHED();
    } else {
      BandAxis a1{gi_.n1, g_.n1, g_.n1, gi_.n1, gp_.h[0], n2h, 1, 1, 0, 0, 0};
      if ((st = band_axis(BAND_DOWN_PROJ, SB, SA, a1, lb1_.dev, l1_.dev, cg, s, "band_proj_axis0")) != ST_OK) return st;
    }
    // K8: c2r on the solve grid (+ <P, AP>)
    const dim3 grid1(row_ctas_);
    const int pk2 = pbeg(dot ? "band_c2r_dot" : "band_c2r",
                         spec_bytes_n() + (dot ? 2.0 : 1.0) * field_bytes(), s);
    if (dot)
      k_c2r_last<R, true><<<grid1, kThreads, smem_rows_, s>>>(SA, y, pdot, partials_, g_, l2_.dev,
                                                              rows_, (R)1, ad, (int)c2r_stage_,
                                                              nullptr);
    else
      k_c2r_last<R, false><<<grid1, kThreads, smem_rows_, s>>>(SA, y, nullptr, nullptr, g_,
                                                               l2_.dev, rows_, (R)1, ad,
                                                               (int)c2r_stage_, nullptr);
    pend(pk2, s);
    FHP_LAUNCHED();
    return ST_OK;
  }

  double spec_bytes_n() const {
    return (double)g_.L * g_.dv * g_.n0 * g_.n1 * g_.n2h * 2 * sizeof(R);
  }

  // A_H via Parseval on the solve grid: W = band(A (X+E)) / prod(B), then
  // A_H[i][j] = <W_i, X_j + E_j>  (exact: X + E is band limited)
  int band_energy(const R* X, int add_macro, double* AH, cudaStream_t s) {
    const size_t n = (size_t)g_.K * g_.L * g_.dv * g_.M;
    R* U = static_cast<R*>(scratch(SCR_BAND_U, n * sizeof(R)));
    R* W = static_cast<R*>(scratch(SCR_BAND_W, n * sizeof(R)));
    if (!U || !W) return ST_OOM;
    if (add_macro) {
      k_add_macro<R><<<grid_for(n), kThreads, 0, s>>>(X, U, g_);
      FHP_LAUNCHED();
    } else {
      FHP_CHECK(cudaMemcpyAsync(U, X, n * sizeof(R), cudaMemcpyDeviceToDevice, s));
    }
    const int proj_saved = gp_.proj;
    const double scale_saved = gp_.scale;
    gp_.proj = 0;
    gp_.scale = 1.0 / (double)gi_.M;
    int st = band_operator(coef_kind_, false, U, nullptr, nullptr, W, nullptr, s, false, false);
    gp_.proj = proj_saved;
    gp_.scale = scale_saved;
    if (st != ST_OK) return st;
    if ((st = cross_dot(W, X, g_, add_macro, (double)g_.M * sizeof(R), s)) != ST_OK) return st;
    return finish_energy(1.0 / (double)g_.M, AH, s);
  }

  int run_operator(int coef, bool pupd, const R* x, R* pio, const R* rvec, R* y, const R* pdot,
                   cudaStream_t s, bool cg, bool dot, bool inproj = false) {
    if (band_) return band_operator(coef, pupd, x, pio, rvec, y, pdot, s, cg, dot, inproj);
    int st;
    if ((st = fwd_passes(coef, pupd, x, pio, rvec, S_, cg, s)) != ST_OK) return st;
    if ((st = proj_pass(S_, cg, s)) != ST_OK) return st;
    return inv_passes(S_, y, (R)(1.0 / (double)g_.M), dot, pdot, cg, s);
  }

  // one CG iteration on all loads (solver.py:124-134), P update fused into pass 1
  int cg_iteration(double* dlog, int log_rows, cudaStream_t s) {
    int st = run_operator(coef_kind_, true, nullptr, p_, r_, ap_, p_, s, true, true, true);
    if (st != ST_OK) return st;
    k_fin_pap<<<dim3(g_.L, g_.K), kThreads, 0, s>>>(partials_, row_ctas_, st_, g_.L,
                                                    1.0 / (double)g_.M, all_done_);
    FHP_LAUNCHED();
    const int pk = pbeg("cg_update", 6.0 * field_bytes(), s);
    // one component per grid row; the parts fit the reduction buffer
    const int C = g_.L * g_.dv;
    const int ux = std::max(1, red_ctas_ / C);
    k_cg_update_comp<R><<<dim3((unsigned)ux, (unsigned)C, (unsigned)g_.K), kThreads, 0, s>>>(
        x_cur_, r_, p_, ap_, partials_, g_, st_, all_done_);
    pend(pk, s);
    FHP_LAUNCHED();
    k_fin_rr<<<dim3(g_.L, g_.K), kThreads, 0, s>>>(partials_, ux * C, st_, g_.L,
                                                   1.0 / (double)g_.M, dlog, log_rows, all_done_);
    FHP_LAUNCHED();
    k_update_all_done<<<1, 1, 0, s>>>(st_, g_.L * g_.K, all_done_);
    FHP_LAUNCHED();
    return ST_OK;
  }

  R* x_cur_ = nullptr;  // the caller's solution buffer during cg_solve
  // potential formulation
  PotParams pp_{};
  R* pe_ = nullptr;            // real fields (L, d) + grid
  cplx<R>* zx_ = nullptr;      // z vectors x, r, p, Ap
  int Tfirst_ = 1;             // column tile of the first-axis pass
  size_t A_elems_ = 0;   // capacity of A_ in elements
  // band representation
  bool band_ = false;
  GridDims gi_{};
  DevLine<R> lb0_, lb1_, lb2_;
  cplx<R>* SB_ = nullptr;
  int brows_ = 1, brow_ctas_ = 1;
  size_t bsmem_rows_ = 0;
  // integration pass kernel: 1 register-resident 512-point lines where they
  // apply (TMA row loads for the full band), 2 the same lines with per-lane
  // cp.async loads, 0 the shared-memory line cores
  int integ_kernel_ = 1;
  int reg512_ctas_per_sm_ = 2;
  int axis_target_mult_ = 1;   // band axis passes: column-tile target x this
  // the solve in progress (cg_begin .. cg_end)
  bool cg_spectral_ = false;
  int cg_proj_ = 1;
  double cg_tol_ = 0.0;
  R* cg_x_ = nullptr;
  double* cg_log_ = nullptr;
  int cg_log_rows_ = 1;
  // spectral CG of band plans
  bool spectral_cg_ = true;
  cplx<R>* zb_ = nullptr;      // z vectors x, r, p, Ap (half spectra of the N grid)
  GridDims gz_{};              // the z vectors as real arrays: M = 2 n0 n1 n2h per comp
  long long projf_parts_ = 0;  // partial sums of the spectral projection pass
};

}  // namespace fhp
