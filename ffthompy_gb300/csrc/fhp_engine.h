// Host-side engine of the Fourier-Galerkin operator: one grid, one precision.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <memory>
#include <string>
#include <vector>

namespace fhp {

// status codes (match include/ffthompy_gb300.h)
enum Status {
  ST_OK = 0,
  ST_NONCONVERGED = 1,
  ST_BREAKDOWN = 2,
  ST_NONFINITE = 3,
  ST_TIMEOUT = 4,
  ST_BAD_ARG = 5,
  ST_OOM = 6,
  ST_CUDA = 7,
};

void set_error(const std::string& msg);
const char* last_error();

// 1D line plan built on the host (long double tables).
struct LinePlanHost {
  int n = 0, nf = 0, blue = 0, nst = 0;
  std::vector<int> rad;                          // core radices
  std::vector<int> pos;                          // n entries (direct lines)
  std::vector<std::complex<long double>> tw;     // nf
  std::vector<std::complex<long double>> chirp;  // n   (Bluestein)
  std::vector<std::complex<long double>> bhat;   // nf  (Bluestein, digit-reversed, / nf)
};
// Scratch slots of EngineBase::scratch; no two users that can be active at
// the same time on one plan share a slot.
enum ScratchSlot {
  SCR_COEF_STAGE = 0,  // host coefficient values staged for conversion
  SCR_LOG,             // CG residual log
  SCR_RHS_TMP,         // macroscopic field of rhs_macro
  SCR_BAND_U,          // band energy: x + E
  SCR_BAND_W,          // band energy: band(A (x + E))
  SCR_HOST_B,          // fhp_homogenize_host: right-hand sides
  SCR_HOST_X,          // fhp_homogenize_host: solution
  SCR_MIX_AX,          // mixed refinement: A x (FP64)
  SCR_MIX_R,           // mixed refinement: residual (FP64)
  SCR_MIX_R32,         // mixed refinement: scaled residual (FP32)
  SCR_MIX_D32,         // mixed refinement: correction (FP32)
  SCR_SOLV_A,          // Richardson / Chebyshev / BiCG vectors
  SCR_SOLV_B,
  SCR_SOLV_C,
  SCR_COEF_STAGE2,     // fhp_homogenize_host_many: the second coefficient upload buffer
  kScratchSlots
};

// two_stage_len: a power-of-two core of exactly this length is factored into
// two stages with the larger radix last (512 = 16 * 32) instead of the default
// ceil(P/4) even stages; 0 = never.
bool build_line_plan(int n, LinePlanHost& out, int two_stage_len = 0);
bool factor_radices(int n, std::vector<int>& rad, int two_stage_len = 0);

// Half spectrum [n0][n1][n2/2+1] (FFT order, FP64) of a ball inclusion's
// exact-integration spectrum from device per-axis tables (fhp_coef.cu); the
// caller transforms it with the plan's inverse_spectrum.
int ball_spectrum(const double* sq, const double* phase, int n0, int n1, int n2, double r,
                  double inv_vol, void* spec, void* stream);

struct PlanConfig {
  int dim = 3;
  int N[3] = {1, 1, 1};      // solve grid (real axes)
  int band[3] = {1, 1, 1};   // grid whose band |k| <= (Nodd-1)/2 carries the projection
  double Y[3] = {1, 1, 1};
  int physics = 0;           // 0 scalar, 1 elasticity, -1 plain FFT plan of ncomp fields
  int ncomp = 1;             // fields of a plain FFT plan
  int nloads = 1;
  double scale = 1.0;        // Ga: prod(2N-1)/prod(N)
  int integ[3] = {0, 0, 0};  // band mode: integration grid (>= 2N-1); 0 = classic
  int ninst = 1;             // cells of the same grid solved together by one plan
};

struct SolveResult {
  std::vector<int> kit;
  std::vector<double> norm_res;
  std::vector<int> status;
  std::vector<double> res_log;  // (log_rows) x L
  int iterations_run = 0;       // max kit
};

// Per-kernel CUDA-event timing of the passes (off unless enabled).
struct ProfEntry {
  std::string name;
  long long launches = 0;
  double ms = 0.0;
  double bytes = 0.0;  // algorithmic bytes per launch
};

struct Profiler {
  bool on = false;
  struct Rec { int kind; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<ProfEntry> kinds;
  std::vector<cudaEvent_t> pool;
  int kind_of(const std::string& name, double bytes);
  void begin(int kind, cudaStream_t s);
  void end(cudaStream_t s);
  void collect();   // synchronises the recorded events
  void reset();
  ~Profiler();
};

class EngineBase {
 public:
  virtual ~EngineBase() = default;
  Profiler prof;
  virtual int precision() const = 0;  // 0: f64, 1: f32
  virtual long long voxels() const = 0;
  virtual int dv() const = 0;
  virtual int loads() const = 0;
  // cells of a batched plan: fields [cell][load][component][grid], per-load
  // results cell-major (cell * loads + load)
  virtual int instances() const = 0;
  // per-load stopping tolerances (cells x loads) for the next CG solve only,
  // in place of its single tol (inner solves of a refinement over cells)
  virtual void set_load_tols(const double* tols, int n) = 0;
  virtual size_t elem_size() const = 0;
  // coefficient (c values per voxel, component-major, f64 on host or device)
  virtual int set_coefficient(int kind, const double* values, bool on_device, cudaStream_t s) = 0;
  // voxels of the coefficient grid per cell (the integration grid of band plans)
  virtual long long coef_voxels() const = 0;
  virtual int coef_kind() const = 0;
  virtual int apply(int proj, const void* x, void* y, cudaStream_t s) = 0;
  // apply with the input projected first (G A G, band plans; same as apply otherwise)
  virtual int apply_ex(int proj, const void* x, void* y, cudaStream_t s, bool inproj) = 0;
  // y += a x (fields of this engine's precision)
  virtual int axpy(double a, const void* x, void* y, cudaStream_t s) = 0;
  // y = G x, G the orthogonal Green projection (no coefficient)
  virtual int project(int proj, const void* x, void* y, cudaStream_t s) = 0;
  virtual int rhs_macro(int proj, void* b, cudaStream_t s) = 0;
  virtual int cg_solve(int proj, const void* b, const void* x0, double tol, int maxiter, void* x,
                       SolveResult& res, int log_cap, cudaStream_t s) = 0;
  // the same solve in phases: cg_begin sets up the state and the first
  // residual, cg_step enqueues one iteration (no host synchronisation; it can
  // be captured into a CUDA graph), cg_done_flag is the device flag that is
  // nonzero once every load has stopped, cg_end finishes and collects the results
  virtual int cg_begin(int proj, const void* b, const void* x0, double tol, int maxiter, void* x,
                       int log_cap, cudaStream_t s) = 0;
  virtual int cg_step(cudaStream_t s) = 0;
  virtual const int* cg_done_flag() const = 0;
  virtual int cg_end(SolveResult& res, cudaStream_t s) = 0;
  // Richardson (kind 0: omega = p0), two-term Chebyshev (kind 1: eigenvalue
  // interval [p0, p1]) and BiCG (kind 2, the transpose operator equal to the
  // operator) over the fused operator, all loads at once with per-load state
  // (ffthompy/general/solver.py:63-77, 142-285)
  virtual int solve_other(int kind, int proj, const void* b, const void* x0, double p0, double p1,
                          double tol, int maxiter, void* x, SolveResult& res, int log_cap,
                          cudaStream_t s) = 0;
  virtual int energy(const void* X, int add_macro, double* AH, cudaStream_t s) = 0;
  // rhs_macro, cg_solve from x0 = 0 (log_cap 1) and energy(x, add_macro = 1)
  // in one call, the driver of applications.py:58-86: b and x are field-sized
  // device buffers, and x holds the solution on return when keep_x is set
  // (an engine may keep the iterates in another form throughout and skip it)
  virtual int homogenize(int proj, double tol, int maxiter, void* b, void* x, bool keep_x,
                         double* AH, SolveResult& res, cudaStream_t s) {
    (void)keep_x;
    int st = rhs_macro(proj, b, s);
    if (st == 0) st = cg_solve(proj, b, nullptr, tol, maxiter, x, res, 1, s);
    if (st == 0) st = energy(x, 1, AH, s);
    return st;
  }
  // grad[c][v] = sum_ij W[i*L+j] dA_H[i][j]/dA_c(v) (W on host, grad FP64 device)
  virtual int energy_gradient(const void* X, int add_macro, const double* W, double* grad,
                              cudaStream_t s) = 0;
  // forward r2c spectrum of X (all comps) into `spec` (natural order, half spectrum)
  virtual int forward_spectrum(const void* x, void* spec, cudaStream_t s) = 0;
  // inverse of a half spectrum into x with scale
  virtual int inverse_spectrum(void* spec, void* x, double scale, cudaStream_t s) = 0;
  virtual size_t spectrum_elems() const = 0;
  virtual const PlanConfig& config() const = 0;
  virtual int pad_spectrum(const void* spec_src, const PlanConfig& src, void* spec_dst,
                           cudaStream_t s) = 0;
  // spec_dst (this grid) = weights * gathered source spectrum (Ga grid-based coefficient)
  virtual int ga_gather(const void* spec_src, const PlanConfig& src, const int* d_index,
                        const double* d_weight, void* spec_dst, cudaStream_t s) = 0;
  // refinement helpers: r = b - ax with per-load sum r^2 (host); dst = s_l*src64;
  // x64 += s_l*d.  d and dst are fields of THIS engine's precision.
  virtual int residual(const void* b, const void* ax, void* r, double* sumsq,
                       cudaStream_t s) = 0;
  virtual int scale_from64(const double* src, const double* scale, void* dst,
                           cudaStream_t s) = 0;
  virtual int add_scaled_to64(const void* d, const double* scale, double* x,
                              cudaStream_t s) = 0;
  // potential formulation (scalar physics, plans without an integration
  // grid; ffthompy/tensorsLowRank/homogenisation.py:41-127).  Potential
  // spectra: 'r' form half spectra of the band grid N, [load][N0][N1][N2/2+1]
  // complex of this engine's precision.
  virtual long long pot_spectrum_elems() const = 0;
  // Persistent per-plan device scratch: slot `slot` holds at least `bytes`
  // (grown with cudaMalloc, never shrunk, freed with the plan), so repeated
  // calls on a plan allocate nothing and plans on other streams share no
  // memory.  nullptr if the allocation fails.
  virtual void* scratch(int slot, size_t bytes) = 0;
  // bh = P B, B_l = div(decrease_N F(A E_l))
  virtual int pot_rhs(void* bh, cudaStream_t s) = 0;
  // yh = P (-div) decrease_N F(A iF(enlarge(grad(P xh))))
  virtual int pot_apply(const void* xh, void* yh, cudaStream_t s) = 0;
  // CG on the preconditioned system with the 'r' Fourier inner product
  virtual int pot_cg(const void* bh, double tol, int maxiter, void* xh, SolveResult& res,
                     int log_cap, cudaStream_t s) = 0;
  // X = iF(enlarge(grad(P xh))): fields (load, comp) on this engine's grid
  virtual int pot_field(const void* xh, void* X, cudaStream_t s) = 0;
  // band plans: CG on the half spectra of the iterates (default) or on the
  // real fields of the solve grid; other plans ignore it
  virtual void set_spectral_cg(bool on) { (void)on; }
  // band plans: integration pass with register-resident lines where they
  // apply (1, default) or the shared-memory line cores (0)
  virtual void set_integration_kernel(int kind) { (void)kind; }
  // time candidate launch shapes of the operator on this plan's buffers and
  // keep the fastest (cached per plan geometry); chosen[3] and best_ms (per
  // application) may be null
  virtual int autotune(cudaStream_t s, int* chosen, float* best_ms) = 0;
  // kernel launch count of the last call (instrumentation)
  long long launches = 0;
};

std::unique_ptr<EngineBase> make_engine_f64(const PlanConfig& cfg, int* status);
std::unique_ptr<EngineBase> make_engine_f32(const PlanConfig& cfg, int* status);

}  // namespace fhp
