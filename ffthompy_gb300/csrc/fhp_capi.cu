// extern "C" entry points of libffthompy_gb300.so (declared in
// include/ffthompy_gb300.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ffthompy_gb300.h"
#include "fhp_engine.h"

struct fhp_plan_s {
  std::unique_ptr<fhp::EngineBase> eng;  // FP64 (F64, MIXED) or FP32 (F32)
  std::unique_ptr<fhp::EngineBase> lo;   // MIXED: FP32 engine of the inner CG
  double eta = 1e-4;                     // MIXED: inner relative tolerance floor
  int max_outer = 30;
  // the plan's own stream for solves requested on the legacy default stream
  // (which cannot be captured into CUDA graphs), and its ordering events
  cudaStream_t own = nullptr;
  cudaEvent_t fence_in = nullptr, fence_out = nullptr;
  // fhp_homogenize_host_many: the upload stream and its two buffers' events
  cudaStream_t copy = nullptr;
  cudaEvent_t copied[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr};
  ~fhp_plan_s() {
    if (own) {
      cudaStreamSynchronize(own);
      cudaStreamDestroy(own);
    }
    if (copy) {
      cudaStreamSynchronize(copy);
      cudaStreamDestroy(copy);
    }
    for (cudaEvent_t e : {fence_in, fence_out, copied[0], copied[1], freed[0], freed[1]})
      if (e) cudaEventDestroy(e);
  }
};

namespace {

int bad(const char* msg) {
  fhp::set_error(msg);
  return FHP_BAD_ARG;
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// per-load results of a plan: loads x cells (cell-major) for a batched plan
int loads_all(const fhp::EngineBase& e) { return e.loads() * e.instances(); }

// entry points that work on one cell only
int one_cell(fhp_plan p) {
  return p && p->eng->instances() != 1 ? bad("the plan is batched over cells; this entry "
                                             "point takes single-cell plans")
                                       : FHP_OK;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FHP_OK;
  fhp::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? FHP_OOM : FHP_CUDA;
}

// A solve requested on the legacy default stream runs on the plan's own
// non-blocking stream instead, so that its iterations can be captured and
// replayed as CUDA graphs: the plan stream first waits for the caller's
// earlier work, and the caller's stream waits for the solve at the end.
class PlanStream {
 public:
  PlanStream(fhp_plan_s* p, cudaStream_t caller) : p_(p), caller_(caller), s_(caller) {
    if (caller != nullptr && caller != cudaStreamLegacy) return;
    if (!p->own) {
      if (cudaStreamCreateWithFlags(&p->own, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&p->fence_in, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&p->fence_out, cudaEventDisableTiming) != cudaSuccess) {
        (void)cudaGetLastError();   // keep the caller's stream (no graphs)
        return;
      }
    }
    if (cudaEventRecord(p->fence_in, caller) != cudaSuccess ||
        cudaStreamWaitEvent(p->own, p->fence_in, 0) != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    s_ = p->own;
  }
  ~PlanStream() {
    if (s_ == caller_) return;
    cudaEventRecord(p_->fence_out, s_);
    cudaStreamWaitEvent(caller_, p_->fence_out, 0);
  }
  cudaStream_t get() const { return s_; }

 private:
  fhp_plan_s* p_;
  cudaStream_t caller_, s_;
};


// The inner tolerance of each cell of a plan of several cells: the cell's own
// min over its active loads, as a plan of that cell alone takes it (the
// FP32 engine's next solve stops each load on its cell's value).
void cell_inner_tols(fhp_plan_s& p, const std::vector<double>& norm,
                     const std::vector<int>& active, double tol) {
  const int K = p.eng->instances(), Lc = p.eng->loads();
  if (K == 1) return;
  std::vector<double> t((size_t)K * Lc, 0.5);
  for (int c = 0; c < K; ++c) {
    double e = 0.5;
    for (int l = c * Lc; l < (c + 1) * Lc; ++l)
      if (active[l]) e = std::min(e, std::max(p.eta, 0.5 * tol / norm[l]));
    for (int l = c * Lc; l < (c + 1) * Lc; ++l) t[l] = e;
  }
  p.lo->set_load_tols(t.data(), K * Lc);
}

// Mixed-precision CG by iterative refinement: the residual r = b - A x is
// formed with the FP64 operator, each load's residual is normalised and solved
// approximately by the FP32 CG (FP64 reductions) to relative tolerance eta,
// and the correction is accumulated in FP64.  Stops per load when
// sqrt(<r,r>) <= tol (the reference's absolute test, solver.py:120-123), when
// the summed inner iterations reach maxiter, or when an outer step stops
// reducing the residual.
int cg_mixed(fhp_plan_s& p, int proj, const void* b, const void* x0, double tol, int maxiter,
             void* xv, fhp::SolveResult& res, int log_rows, cudaStream_t s) {
  fhp::EngineBase& hi = *p.eng;
  fhp::EngineBase& lo = *p.lo;
  const int L = loads_all(hi);
  const double M = (double)hi.voxels();
  const size_t n = (size_t)L * hi.dv() * hi.voxels();
  double* x = static_cast<double*>(xv);
  // the plan's persistent scratch: nothing is allocated per solve
  void* ax = hi.scratch(fhp::SCR_MIX_AX, n * 8);
  void* r = hi.scratch(fhp::SCR_MIX_R, n * 8);
  void* r32 = hi.scratch(fhp::SCR_MIX_R32, n * 4);
  void* d32 = hi.scratch(fhp::SCR_MIX_D32, n * 4);
  int st = (ax && r && r32 && d32) ? FHP_OK : FHP_OOM;
  std::vector<double> sumsq(L), norm(L), sc_in(L), sc_out(L);
  std::vector<int> kit(L, 0), status(L, 0), active(L, 1);
  res.res_log.assign((size_t)std::max(1, log_rows) * L, 0.0);
  if (st == FHP_OK) {
    if (x0) {
      st = cuda_status(cudaMemcpyAsync(x, x0, n * 8, cudaMemcpyDeviceToDevice, s), "copy");
      if (st == FHP_OK) st = hi.apply_ex(proj, x, ax, s, true);
    } else {
      st = cuda_status(cudaMemsetAsync(x, 0, n * 8, s), "memset");
      if (st == FHP_OK) st = cuda_status(cudaMemsetAsync(ax, 0, n * 8, s), "memset");
    }
  }
  if (st == FHP_OK) st = hi.residual(b, ax, r, sumsq.data(), s);
  for (int l = 0; l < L; ++l) {
    norm[l] = std::sqrt(sumsq[l] / M);
    res.res_log[l] = norm[l];
    if (!std::isfinite(norm[l])) { status[l] = FHP_NONFINITE; active[l] = 0; }
    if (!(norm[l] > tol && maxiter > 0)) active[l] = 0;
  }
  for (int outer = 0; st == FHP_OK && outer < p.max_outer; ++outer) {
    int any = 0, room = maxiter;
    double eta = 0.5;
    for (int l = 0; l < L; ++l) {
      if (!active[l]) continue;
      any = 1;
      room = std::min(room, maxiter - kit[l]);
      eta = std::min(eta, std::max(p.eta, 0.5 * tol / norm[l]));
    }
    if (!any || room <= 0) break;
    for (int l = 0; l < L; ++l) {
      sc_in[l] = active[l] ? 1.0 / norm[l] : 0.0;
      sc_out[l] = active[l] ? norm[l] : 0.0;
    }
    if ((st = lo.scale_from64(static_cast<const double*>(r), sc_in.data(), r32, s)) != FHP_OK) break;
    cell_inner_tols(p, norm, active, tol);
    fhp::SolveResult in;
    if ((st = lo.cg_solve(proj, r32, nullptr, eta, room, d32, in, 1, s)) != FHP_OK) break;
    // x += G (s d): the FP32 correction carries roundoff outside range(G),
    // invisible to the residual but first order in the energy, so it is
    // projected in FP64 before it is accumulated (d32 holds FP32 values: the
    // FP32 engine owns the matching kernel instance)
    if ((st = cuda_status(cudaMemsetAsync(ax, 0, n * 8, s), "memset")) != FHP_OK) break;
    if ((st = lo.add_scaled_to64(d32, sc_out.data(), static_cast<double*>(ax), s)) != FHP_OK) break;
    if ((st = hi.project(proj, ax, r, s)) != FHP_OK) break;
    if ((st = hi.axpy(1.0, r, x, s)) != FHP_OK) break;
    if ((st = hi.apply_ex(proj, x, ax, s, true)) != FHP_OK) break;
    if ((st = hi.residual(b, ax, r, sumsq.data(), s)) != FHP_OK) break;
    for (int l = 0; l < L; ++l) {
      if (!active[l]) continue;
      const double prev = norm[l];
      kit[l] += in.kit[l];
      norm[l] = std::sqrt(sumsq[l] / M);
      if (kit[l] < log_rows) res.res_log[(size_t)kit[l] * L + l] = norm[l];
      if (!std::isfinite(norm[l])) { status[l] = FHP_NONFINITE; active[l] = 0; continue; }
      if (norm[l] <= tol) { active[l] = 0; continue; }
      if (kit[l] >= maxiter || in.kit[l] == 0 || norm[l] > 0.5 * prev) {
        status[l] = FHP_NONCONVERGED;  // stagnation of the refinement
        active[l] = 0;
      }
    }
  }
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  res.kit = kit;
  res.norm_res.resize(L);
  res.status = status;
  res.iterations_run = 0;
  for (int l = 0; l < L; ++l) {
    res.norm_res[l] = kit[l] == 0 ? 0.0 : norm[l];
    if (status[l] == 0 && norm[l] > tol && kit[l] > 0) res.status[l] = FHP_NONCONVERGED;
    res.iterations_run = std::max(res.iterations_run, kit[l]);
  }
  return st;
}

// done[i] = *flags[i] for the plans of the current graph, all_done = AND
__global__ void k_gather_done(const int* const* __restrict__ flags, const int* __restrict__ idx,
                              int n, int* __restrict__ done, int* all_done) {
  int d = 1;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int v = *flags[idx[i]];
    done[i] = v;
    d &= v;
  }
  d = __syncthreads_and(d);
  if (threadIdx.x == 0) *all_done = d;
}

// Several plans' CG solves advanced together (fhp_cg_solve_many).  Each plan
// keeps its own loads, scalars and stopping tests (cg_begin / cg_end).  One
// iteration of each plan is captured once as its own graph; the iteration of
// the ensemble is a graph whose nodes are these child graphs of the plans
// still running, all independent (the GPU runs them side by side), followed
// by one kernel that gathers the plans' done flags.  The host reads them every
// few iterations and, once a quarter of the graph's plans have stopped,
// assembles a new graph of the running ones (a stopped plan's kernels would
// still be launched, only to return).  Without graph capture (profiling on,
// or a refused capture) the running plans' iterations are launched directly.
int cg_many(const std::vector<fhp::EngineBase*>& engs, int proj, const std::vector<const void*>& b,
            const std::vector<double>& tol, int maxiter, const std::vector<void*>& x,
            std::vector<fhp::SolveResult>& res, cudaStream_t s) {
  const int n = (int)engs.size();
  res.assign(n, fhp::SolveResult());
  if (n == 0) return FHP_OK;
  int st = FHP_OK;
  for (int i = 0; i < n && st == FHP_OK; ++i)
    st = engs[i]->cg_begin(proj, b[i], nullptr, tol[i], maxiter, x[i], 1, s);
  if (st != FHP_OK) return st;
  std::vector<const int*> hflags(n);
  bool prof = false;
  for (int i = 0; i < n; ++i) {
    hflags[i] = engs[i]->cg_done_flag();
    prof = prof || engs[i]->prof.on;
  }
  const int** dflags = nullptr;
  int *didx = nullptr, *ddone = nullptr, *hdone = nullptr;
  std::vector<cudaGraph_t> child(n, nullptr);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::vector<long long> per_iter(n, 0);
  auto drop_graph = [&]() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
  };
  auto cleanup = [&]() {
    drop_graph();
    for (cudaGraph_t c : child)
      if (c) cudaGraphDestroy(c);
    if (dflags) cudaFreeAsync(dflags, s);
    if (didx) cudaFreeAsync(didx, s);
    if (ddone) cudaFreeAsync(ddone, s);
    if (hdone) cudaFreeHost(hdone);
  };
  // running plans (indices into engs); ddone[0..m) their flags, ddone[n] the AND
  std::vector<int> run(n);
  for (int i = 0; i < n; ++i) run[i] = i;
  st = cuda_status(cudaMallocAsync((void**)&dflags, n * sizeof(int*), s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocAsync((void**)&didx, n * sizeof(int), s), "alloc");
  if (st == FHP_OK)
    st = cuda_status(cudaMallocAsync((void**)&ddone, (n + 1) * sizeof(int), s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocHost((void**)&hdone, (n + 1) * sizeof(int)), "alloc");
  if (st == FHP_OK)
    st = cuda_status(cudaMemcpyAsync(dflags, hflags.data(), n * sizeof(int*),
                                     cudaMemcpyHostToDevice, s), "copy");
  // the host vector must outlive the copy from pageable memory
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  if (st != FHP_OK) { cleanup(); return st; }
  // one iteration of every plan as its own graph
  bool use_graph = !prof && maxiter > 0;
  for (int i = 0; i < n && use_graph && st == FHP_OK; ++i) {
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      use_graph = false;
      break;
    }
    const long long l0 = engs[i]->launches;
    const int cst = engs[i]->cg_step(s);
    per_iter[i] = engs[i]->launches - l0;
    engs[i]->launches = l0;
    const cudaError_t e = cudaStreamEndCapture(s, &child[i]);
    if (cst != FHP_OK) st = cst;
    if (e != cudaSuccess || !child[i]) use_graph = false;
  }
  (void)cudaGetLastError();  // a refused capture leaves no error behind
  if (st != FHP_OK) { cleanup(); return st; }
  // the ensemble's iteration: the running plans' graphs, then the gather
  int gm = 0;
  auto build_graph = [&]() {
    drop_graph();
    if (!use_graph) return;
    bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess;
    std::vector<cudaGraphNode_t> nodes(run.size());
    for (size_t j = 0; j < run.size() && ok; ++j)
      ok = cudaGraphAddChildGraphNode(&nodes[j], graph, nullptr, 0, child[run[j]]) == cudaSuccess;
    gm = (int)run.size();
    int* dall = ddone + n;
    void* args[] = {(void*)&dflags, (void*)&didx, (void*)&gm, (void*)&ddone, (void*)&dall};
    cudaKernelNodeParams kp = {};
    kp.func = (void*)k_gather_done;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(256);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    cudaGraphNode_t kn;
    if (ok) ok = cudaGraphAddKernelNode(&kn, graph, nodes.data(), nodes.size(), &kp) == cudaSuccess;
    if (ok) ok = cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess;
    if (!ok) {
      drop_graph();
      use_graph = false;
    }
    (void)cudaGetLastError();
  };
  auto upload_run = [&]() {
    int r = cuda_status(cudaMemcpyAsync(didx, run.data(), run.size() * sizeof(int),
                                        cudaMemcpyHostToDevice, s), "copy");
    if (r == FHP_OK) r = cuda_status(cudaStreamSynchronize(s), "sync");
    return r;
  };
  st = upload_run();
  if (st == FHP_OK) build_graph();
  std::vector<int> gset = run;   // the plans of the graph, in the order of its done flags
  int done_iters = 0, chunk = 2;
  bool first = true;
  while (st == FHP_OK && done_iters < maxiter) {
    // the done flags of the graph's plans (refreshed by its last node), or
    // gathered here for direct launches and before the first iteration
    const bool gathered_here = first || !gexec;
    const std::vector<int>& order = gathered_here ? run : gset;
    if (gathered_here) {
      if (!first && (st = upload_run()) != FHP_OK) break;
      k_gather_done<<<1, 256, 0, s>>>(dflags, didx, (int)run.size(), ddone, ddone + n);
      st = cuda_status(cudaGetLastError(), "k_gather_done");
      if (st != FHP_OK) break;
    }
    st = cuda_status(cudaMemcpyAsync(hdone, ddone, (n + 1) * sizeof(int), cudaMemcpyDeviceToHost,
                                     s), "copy");
    if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
    if (st != FHP_OK) break;
    first = false;
    if (hdone[n]) break;
    std::vector<int> still;
    for (size_t j = 0; j < order.size(); ++j)
      if (!hdone[j]) still.push_back(order[j]);
    if (still.empty()) break;
    run.swap(still);
    if (gexec && 4 * run.size() <= 3 * gset.size()) {
      // a quarter of the graph's plans have stopped: a graph of the running ones
      if ((st = upload_run()) != FHP_OK) break;
      build_graph();
      gset = run;
    }
    const int nit = std::min(chunk, maxiter - done_iters);
    for (int it = 0; it < nit && st == FHP_OK; ++it) {
      if (gexec) {
        st = cuda_status(cudaGraphLaunch(gexec, s), "cudaGraphLaunch");
        for (int j : gset) engs[j]->launches += per_iter[j];
      } else {
        for (size_t j = 0; j < run.size() && st == FHP_OK; ++j) st = engs[run[j]]->cg_step(s);
      }
    }
    done_iters += nit;
    chunk = std::min(chunk * 2, 16);
  }
  for (int i = 0; i < n && st == FHP_OK; ++i) st = engs[i]->cg_end(res[i], s);
  cleanup();
  return st;
}

// Mixed precision over several plans: the refinement of cg_mixed per plan,
// with each outer step's FP32 inner solves of all plans advanced together.
int cg_mixed_many(const std::vector<fhp_plan_s*>& plans, int proj,
                  const std::vector<const void*>& b, double tol, int maxiter,
                  const std::vector<void*>& xv, std::vector<fhp::SolveResult>& out,
                  cudaStream_t s) {
  const int n = (int)plans.size();
  out.assign(n, fhp::SolveResult());
  struct P {
    void *ax, *r, *r32, *d32;
    std::vector<double> sumsq, norm, sc_in, sc_out;
    std::vector<int> kit, status, active;
  };
  std::vector<P> ps(n);
  int st = FHP_OK;
  for (int i = 0; i < n && st == FHP_OK; ++i) {
    fhp::EngineBase& hi = *plans[i]->eng;
    const int L = loads_all(hi);
    const size_t nv = (size_t)L * hi.dv() * hi.voxels();
    P& q = ps[i];
    q.ax = hi.scratch(fhp::SCR_MIX_AX, nv * 8);
    q.r = hi.scratch(fhp::SCR_MIX_R, nv * 8);
    q.r32 = hi.scratch(fhp::SCR_MIX_R32, nv * 4);
    q.d32 = hi.scratch(fhp::SCR_MIX_D32, nv * 4);
    if (!(q.ax && q.r && q.r32 && q.d32)) { st = FHP_OOM; break; }
    q.sumsq.assign(L, 0.);
    q.norm.assign(L, 0.);
    q.sc_in.assign(L, 0.);
    q.sc_out.assign(L, 0.);
    q.kit.assign(L, 0);
    q.status.assign(L, 0);
    q.active.assign(L, 1);
    st = cuda_status(cudaMemsetAsync(xv[i], 0, nv * 8, s), "memset");
    if (st == FHP_OK) st = cuda_status(cudaMemsetAsync(q.ax, 0, nv * 8, s), "memset");
    if (st == FHP_OK) st = hi.residual(b[i], q.ax, q.r, q.sumsq.data(), s);
    const double M = (double)hi.voxels();
    for (int l = 0; l < L; ++l) {
      q.norm[l] = std::sqrt(q.sumsq[l] / M);
      if (!std::isfinite(q.norm[l])) { q.status[l] = FHP_NONFINITE; q.active[l] = 0; }
      if (!(q.norm[l] > tol && maxiter > 0)) q.active[l] = 0;
    }
  }
  const int max_outer = n ? plans[0]->max_outer : 0;
  for (int outer = 0; st == FHP_OK && outer < max_outer; ++outer) {
    std::vector<fhp::EngineBase*> lo;
    std::vector<const void*> rb;
    std::vector<void*> dx;
    std::vector<double> eta;
    std::vector<int> idx;
    int room = maxiter;
    for (int i = 0; i < n; ++i) {
      P& q = ps[i];
      const int L = (int)q.kit.size();
      int any = 0;
      double e = 0.5;
      for (int l = 0; l < L; ++l) {
        if (!q.active[l]) continue;
        any = 1;
        room = std::min(room, maxiter - q.kit[l]);
        e = std::min(e, std::max(plans[i]->eta, 0.5 * tol / q.norm[l]));
      }
      if (!any) continue;
      for (int l = 0; l < L; ++l) {
        q.sc_in[l] = q.active[l] ? 1.0 / q.norm[l] : 0.0;
        q.sc_out[l] = q.active[l] ? q.norm[l] : 0.0;
      }
      if ((st = plans[i]->lo->scale_from64(static_cast<const double*>(q.r), q.sc_in.data(), q.r32,
                                           s)) != FHP_OK) break;
      cell_inner_tols(*plans[i], q.norm, q.active, tol);
      lo.push_back(plans[i]->lo.get());
      rb.push_back(q.r32);
      dx.push_back(q.d32);
      eta.push_back(e);
      idx.push_back(i);
    }
    if (st != FHP_OK || idx.empty() || room <= 0) break;
    std::vector<fhp::SolveResult> in;
    if ((st = cg_many(lo, proj, rb, eta, room, dx, in, s)) != FHP_OK) break;
    for (size_t j = 0; j < idx.size() && st == FHP_OK; ++j) {
      const int i = idx[j];
      fhp::EngineBase& hi = *plans[i]->eng;
      P& q = ps[i];
      double* x = static_cast<double*>(xv[i]);
      const size_t nv = (size_t)loads_all(hi) * hi.dv() * hi.voxels();
      const double M = (double)hi.voxels();
      // x += G (s d), as cg_mixed
      if ((st = cuda_status(cudaMemsetAsync(q.ax, 0, nv * 8, s), "memset")) != FHP_OK) break;
      if ((st = plans[i]->lo->add_scaled_to64(q.d32, q.sc_out.data(), static_cast<double*>(q.ax),
                                              s)) != FHP_OK) break;
      if ((st = hi.project(proj, q.ax, q.r, s)) != FHP_OK) break;
      if ((st = hi.axpy(1.0, q.r, x, s)) != FHP_OK) break;
      if ((st = hi.apply_ex(proj, x, q.ax, s, true)) != FHP_OK) break;
      if ((st = hi.residual(b[i], q.ax, q.r, q.sumsq.data(), s)) != FHP_OK) break;
      for (int l = 0; l < (int)q.kit.size(); ++l) {
        if (!q.active[l]) continue;
        const double prev = q.norm[l];
        q.kit[l] += in[j].kit[l];
        q.norm[l] = std::sqrt(q.sumsq[l] / M);
        if (!std::isfinite(q.norm[l])) { q.status[l] = FHP_NONFINITE; q.active[l] = 0; continue; }
        if (q.norm[l] <= tol) { q.active[l] = 0; continue; }
        if (q.kit[l] >= maxiter || in[j].kit[l] == 0 || q.norm[l] > 0.5 * prev) {
          q.status[l] = FHP_NONCONVERGED;
          q.active[l] = 0;
        }
      }
    }
  }
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  for (int i = 0; i < n; ++i) {
    P& q = ps[i];
    fhp::SolveResult& r = out[i];
    const int L = (int)q.kit.size();
    r.kit = q.kit;
    r.status = q.status;
    r.norm_res.assign(L, 0.);
    r.res_log.assign(L, 0.);
    for (int l = 0; l < L; ++l) {
      r.norm_res[l] = q.kit[l] == 0 ? 0.0 : q.norm[l];
      if (r.status[l] == 0 && q.norm[l] > tol && q.kit[l] > 0) r.status[l] = FHP_NONCONVERGED;
      r.iterations_run = std::max(r.iterations_run, q.kit[l]);
    }
  }
  return st;
}

}  // namespace

extern "C" {

int fhp_version(void) { return 100; }

const char* fhp_status_string(int status) {
  switch (status) {
    case FHP_OK: return "ok";
    case FHP_NONCONVERGED: return "not converged (maxiter reached)";
    case FHP_BREAKDOWN: return "CG breakdown (<P,AP> <= 0)";
    case FHP_NONFINITE: return "non-finite value in a reduction";
    case FHP_TIMEOUT: return "timeout";
    case FHP_BAD_ARG: return "bad argument";
    case FHP_OOM: return "out of device memory";
    case FHP_CUDA: return "CUDA error";
    default: return "unknown status";
  }
}

const char* fhp_last_error(void) { return fhp::last_error(); }

namespace {
int plan_create(fhp_plan* out, int dim, const int* n, const int* n_band, const double* Y,
                int physics, int nloads, double g_scale, int precision, int ncells) {
  if (!out) return bad("out is NULL");
  *out = nullptr;
  if (dim != 2 && dim != 3) return bad("dim must be 2 or 3");
  if (!n || !n_band || !Y) return bad("n, n_band and Y are required");
  if (physics != FHP_SCALAR && physics != FHP_ELASTICITY) return bad("unknown physics");
  if (!(g_scale > 0) || !std::isfinite(g_scale)) return bad("g_scale must be positive");
  fhp::PlanConfig cfg;
  cfg.dim = dim;
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1 || n_band[i] < 1 || n_band[i] > n[i]) return bad("bad grid sizes");
    if (n[i] > 4096) return bad("grid size per axis must be <= 4096");
    cfg.N[i] = n[i];
    cfg.band[i] = n_band[i];
    cfg.Y[i] = Y[i];
  }
  cfg.physics = physics;
  cfg.nloads = nloads;
  cfg.scale = g_scale;
  cfg.ninst = ncells;
  int st = FHP_OK;
  std::unique_ptr<fhp::EngineBase> e, lo;
  if (precision == FHP_F64 || precision == FHP_MIXED) e = fhp::make_engine_f64(cfg, &st);
  else if (precision == FHP_F32) e = fhp::make_engine_f32(cfg, &st);
  else return bad("unknown precision");
  if (!e) return st == FHP_OK ? FHP_CUDA : st;
  if (precision == FHP_MIXED) {
    lo = fhp::make_engine_f32(cfg, &st);
    if (!lo) return st == FHP_OK ? FHP_CUDA : st;
  }
  auto* p = new (std::nothrow) fhp_plan_s;
  if (!p) return FHP_OOM;
  p->eng = std::move(e);
  p->lo = std::move(lo);
  *out = p;
  return FHP_OK;
}
}  // namespace

int fhp_plan_create(fhp_plan* out, int dim, const int* n, const int* n_band, const double* Y,
                    int physics, int nloads, double g_scale, int precision) {
  return plan_create(out, dim, n, n_band, Y, physics, nloads, g_scale, precision, 1);
}

int fhp_plan_create_cells(fhp_plan* out, int dim, const int* n, const int* n_band,
                          const double* Y, int physics, int nloads, double g_scale,
                          int precision, int ncells) {
  if (ncells < 1 || ncells > 65535) return bad("ncells must be in 1..65535");
  return plan_create(out, dim, n, n_band, Y, physics, nloads, g_scale, precision, ncells);
}

int fhp_plan_cells(fhp_plan plan) { return plan ? plan->eng->instances() : 0; }

int fhp_plan_create_band(fhp_plan* out, int dim, const int* n, const int* n_int,
                         const double* Y, int physics, int nloads, double g_scale,
                         int precision) {
  if (!out) return bad("out is NULL");
  *out = nullptr;
  if (dim != 2 && dim != 3) return bad("dim must be 2 or 3");
  if (!n || !n_int || !Y) return bad("n, n_int and Y are required");
  if (physics != FHP_SCALAR && physics != FHP_ELASTICITY) return bad("unknown physics");
  if (!(g_scale > 0) || !std::isfinite(g_scale)) return bad("g_scale must be positive");
  fhp::PlanConfig cfg;
  cfg.dim = dim;
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1 || n[i] > 4096 || n_int[i] > 4096) return bad("bad grid sizes");
    if (n_int[i] < 2 * n[i] - 1) return bad("integration grid must be >= 2n-1");
    cfg.N[i] = n[i];
    cfg.band[i] = n[i];
    cfg.integ[i] = n_int[i];
    cfg.Y[i] = Y[i];
  }
  cfg.physics = physics;
  cfg.nloads = nloads;
  cfg.scale = g_scale;
  int st = FHP_OK;
  std::unique_ptr<fhp::EngineBase> e, lo;
  if (precision == FHP_F64 || precision == FHP_MIXED) e = fhp::make_engine_f64(cfg, &st);
  else if (precision == FHP_F32) e = fhp::make_engine_f32(cfg, &st);
  else return bad("unknown precision");
  if (!e) return st == FHP_OK ? FHP_CUDA : st;
  if (precision == FHP_MIXED) {
    lo = fhp::make_engine_f32(cfg, &st);
    if (!lo) return st == FHP_OK ? FHP_CUDA : st;
  }
  auto* p = new (std::nothrow) fhp_plan_s;
  if (!p) return FHP_OOM;
  p->eng = std::move(e);
  p->lo = std::move(lo);
  *out = p;
  return FHP_OK;
}

int fhp_plan_set_refinement(fhp_plan plan, double eta, int max_outer) {
  if (!plan || !plan->lo) return bad("refinement parameters apply to FHP_MIXED plans");
  if (!(eta > 0 && eta < 1) || max_outer < 1) return bad("need 0 < eta < 1, max_outer >= 1");
  plan->eta = eta;
  plan->max_outer = max_outer;
  return FHP_OK;
}

int fhp_plan_set_band_cg(fhp_plan plan, int spectral) {
  if (!plan) return bad("plan is NULL");
  if (spectral != 0 && spectral != 1) return bad("spectral must be 0 or 1");
  plan->eng->set_spectral_cg(spectral != 0);
  if (plan->lo) plan->lo->set_spectral_cg(spectral != 0);
  return FHP_OK;
}

int fhp_plan_set_integration_kernel(fhp_plan plan, int kind) {
  if (!plan) return bad("plan is NULL");
  if (kind < 0 || kind > 2) return bad("kind must be 0, 1 or 2");
  plan->eng->set_integration_kernel(kind);
  if (plan->lo) plan->lo->set_integration_kernel(kind);
  return FHP_OK;
}

int fhp_plan_autotune(fhp_plan plan, int* chosen, float* ms_per_apply, void* stream) {
  if (!plan) return bad("plan is NULL");
  cudaStream_t s = as_stream(stream);
  int st = plan->eng->autotune(s, chosen, ms_per_apply);
  if (st == FHP_OK && plan->lo) st = plan->lo->autotune(s, nullptr, nullptr);
  return st;
}

int fhp_plan_destroy(fhp_plan plan) {
  delete plan;
  return FHP_OK;
}

int fhp_plan_query(fhp_plan plan, long long* voxels, int* components, int* loads,
                   int* elem_bytes) {
  if (!plan) return bad("plan is NULL");
  if (voxels) *voxels = plan->eng->voxels();
  if (components) *components = plan->eng->dv();
  if (loads) *loads = plan->eng->loads();
  if (elem_bytes) *elem_bytes = (int)plan->eng->elem_size();
  return FHP_OK;
}

int fhp_set_coefficient(fhp_plan plan, int kind, const double* values, int on_device,
                        void* stream) {
  if (!plan || !values) return bad("plan and values are required");
  int st = plan->eng->set_coefficient(kind, values, on_device != 0, as_stream(stream));
  if (st == FHP_OK && plan->lo)
    st = plan->lo->set_coefficient(kind, values, on_device != 0, as_stream(stream));
  return st;
}

int fhp_apply(fhp_plan plan, int proj, const void* x, void* y, void* stream) {
  if (!plan || !x || !y) return bad("plan, x and y are required");
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  return plan->eng->apply(proj, x, y, as_stream(stream));
}

int fhp_rhs_macro(fhp_plan plan, int proj, void* b, void* stream) {
  if (!plan || !b) return bad("plan and b are required");
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  return plan->eng->rhs_macro(proj, b, as_stream(stream));
}

int fhp_potential_rhs(fhp_plan plan, void* bh, void* stream) {
  if (!plan || !bh) return bad("plan and bh are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  return plan->eng->pot_rhs(bh, as_stream(stream));
}

int fhp_potential_apply(fhp_plan plan, const void* xh, void* yh, void* stream) {
  if (!plan || !xh || !yh) return bad("plan, xh and yh are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  return plan->eng->pot_apply(xh, yh, as_stream(stream));
}

int fhp_potential_cg(fhp_plan plan, const void* bh, double tol, int maxiter, void* xh, int* kit,
                     double* norm_res, int* status, double* res_log, int log_rows,
                     void* stream) {
  if (!plan || !bh || !xh) return bad("plan, bh and xh are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  if (maxiter < 0) return bad("maxiter must be >= 0");
  if (!(tol >= 0)) return bad("tol must be >= 0");
  fhp::SolveResult r;
  const int rows = res_log ? std::max(1, log_rows) : 1;
  int st = plan->eng->pot_cg(bh, tol, maxiter, xh, r, rows, as_stream(stream));
  if (st != FHP_OK) return st;
  const int L = plan->eng->loads();
  for (int l = 0; l < L && l < (int)r.kit.size(); ++l) {
    if (kit) kit[l] = r.kit[l];
    if (norm_res) norm_res[l] = r.norm_res[l];
    if (status) status[l] = r.status[l];
  }
  if (res_log && !r.res_log.empty())
    std::memcpy(res_log, r.res_log.data(),
                std::min<size_t>((size_t)rows * L, r.res_log.size()) * sizeof(double));
  return FHP_OK;
}

int fhp_potential_field(fhp_plan plan, const void* xh, void* X, void* stream) {
  if (!plan || !xh || !X) return bad("plan, xh and X are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  return plan->eng->pot_field(xh, X, as_stream(stream));
}

int fhp_cg_solve(fhp_plan plan, int proj, const void* b, const void* x0, double tol,
                 int maxiter, void* x, int* kit, double* norm_res, int* status,
                 double* res_log, int log_rows, void* stream) {
  if (!plan || !b || !x) return bad("plan, b and x are required");
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  if (maxiter < 0) return bad("maxiter must be >= 0");
  if (!(tol >= 0)) return bad("tol must be >= 0");
  fhp::SolveResult r;
  const int rows = res_log ? std::max(1, log_rows) : 1;
  int st;
  {
    PlanStream ps(plan, as_stream(stream));
    st = plan->lo ? cg_mixed(*plan, proj, b, x0, tol, maxiter, x, r, rows, ps.get())
                  : plan->eng->cg_solve(proj, b, x0, tol, maxiter, x, r, rows, ps.get());
  }
  if (st != FHP_OK && r.kit.empty()) return st;
  const int L = loads_all(*plan->eng);
  for (int l = 0; l < L && l < (int)r.kit.size(); ++l) {
    if (kit) kit[l] = r.kit[l];
    if (norm_res) norm_res[l] = r.norm_res[l];
    if (status) status[l] = r.status[l];
  }
  if (res_log && !r.res_log.empty())
    std::memcpy(res_log, r.res_log.data(),
                std::min<size_t>((size_t)rows * L, r.res_log.size()) * sizeof(double));
  return st;
}

int fhp_cg_solve_many(int count, const fhp_plan* plans, int proj, const void* const* b,
                      double tol, int maxiter, void* const* x, int* kit, double* norm_res,
                      int* status, void* stream) {
  if (count < 0 || (count > 0 && (!plans || !b || !x))) return bad("plans, b and x are required");
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  if (maxiter < 0) return bad("maxiter must be >= 0");
  if (!(tol >= 0)) return bad("tol must be >= 0");
  if (count == 0) return FHP_OK;
  const bool mixed = plans[0] && plans[0]->lo;
  for (int i = 0; i < count; ++i) {
    if (!plans[i] || !b[i] || !x[i]) return bad("every plan needs a plan, b and x");
    if ((plans[i]->lo != nullptr) != mixed) return bad("plans mix FHP_MIXED and other precisions");
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return bad("a plan appears twice");
  }
  PlanStream pstream(plans[0], as_stream(stream));
  cudaStream_t s = pstream.get();
  std::vector<fhp::SolveResult> r;
  std::vector<const void*> bv(b, b + count);
  std::vector<void*> xv(x, x + count);
  int st;
  if (mixed) {
    std::vector<fhp_plan_s*> ps(plans, plans + count);
    st = cg_mixed_many(ps, proj, bv, tol, maxiter, xv, r, s);
  } else {
    std::vector<fhp::EngineBase*> engs(count);
    for (int i = 0; i < count; ++i) engs[i] = plans[i]->eng.get();
    st = cg_many(engs, proj, bv, std::vector<double>(count, tol), maxiter, xv, r, s);
  }
  int off = 0;
  for (int i = 0; i < count; ++i) {
    const int L = loads_all(*plans[i]->eng);
    for (int l = 0; l < L && i < (int)r.size() && l < (int)r[i].kit.size(); ++l) {
      if (kit) kit[off + l] = r[i].kit[l];
      if (norm_res) norm_res[off + l] = r[i].norm_res[l];
      if (status) status[off + l] = r[i].status[l];
    }
    off += L;
  }
  return st;
}

namespace {
int solve_other_c(int kind, fhp_plan plan, int proj, const void* b, const void* x0, double p0,
                  double p1, double tol, int maxiter, void* x, int* kit, double* norm_res,
                  int* status, void* stream) {
  if (!plan || !b || !x) return bad("plan, b and x are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  if (maxiter < 0) return bad("maxiter must be >= 0");
  if (!(tol >= 0)) return bad("tol must be >= 0");
  fhp::SolveResult r;
  PlanStream ps(plan, as_stream(stream));
  const int st = plan->eng->solve_other(kind, proj, b, x0, p0, p1, tol, maxiter, x, r, 1,
                                        ps.get());
  const int L = plan->eng->loads();
  for (int l = 0; l < L && l < (int)r.kit.size(); ++l) {
    if (kit) kit[l] = r.kit[l];
    if (norm_res) norm_res[l] = r.norm_res[l];
    if (status) status[l] = r.status[l];
  }
  return st;
}
}  // namespace

int fhp_richardson_solve(fhp_plan plan, int proj, const void* b, const void* x0, double omega,
                         double tol, int maxiter, void* x, int* kit, double* norm_res,
                         int* status, void* stream) {
  if (!(omega > 0)) return bad("omega must be > 0");
  return solve_other_c(0, plan, proj, b, x0, omega, 0., tol, maxiter, x, kit, norm_res, status,
                       stream);
}

int fhp_chebyshev_solve(fhp_plan plan, int proj, const void* b, const void* x0, double eig_min,
                        double eig_max, double tol, int maxiter, void* x, int* kit,
                        double* norm_res, int* status, void* stream) {
  if (!(eig_max > eig_min && eig_min > 0)) return bad("need 0 < eig_min < eig_max");
  return solve_other_c(1, plan, proj, b, x0, eig_min, eig_max, tol, maxiter, x, kit, norm_res,
                       status, stream);
}

int fhp_bicg_solve(fhp_plan plan, int proj, const void* b, const void* x0, double tol,
                   int maxiter, void* x, int* kit, double* norm_res, int* status, void* stream) {
  return solve_other_c(2, plan, proj, b, x0, 0., 0., tol, maxiter, x, kit, norm_res, status,
                       stream);
}

int fhp_energy_matrix(fhp_plan plan, const void* X, int add_macro, double* AH, void* stream) {
  if (!plan || !X || !AH) return bad("plan, X and AH are required");
  return plan->eng->energy(X, add_macro, AH, as_stream(stream));
}

int fhp_energy_gradient(fhp_plan plan, const void* X, int add_macro, const double* W,
                        double* grad, void* stream) {
  if (!plan || !X || !W || !grad) return bad("plan, X, W and grad are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  return plan->eng->energy_gradient(X, add_macro, W, grad, as_stream(stream));
}

int fhp_fourier_interp(fhp_plan src, fhp_plan dst, const void* x_src, void* x_dst,
                       void* stream) {
  if (!src || !dst || !x_src || !x_dst) return bad("plans and fields are required");
  if (one_cell(src) || one_cell(dst)) return FHP_BAD_ARG;
  const fhp::PlanConfig& a = src->eng->config();
  const fhp::PlanConfig& b = dst->eng->config();
  if (a.dim != b.dim || src->eng->dv() * src->eng->loads() != dst->eng->dv() * dst->eng->loads() ||
      src->eng->precision() != dst->eng->precision())
    return bad("plans differ in dim, field count or precision");
  for (int i = 0; i < a.dim; ++i)
    if (b.N[i] < a.N[i]) return bad("destination grid must not be smaller");
  cudaStream_t s = as_stream(stream);
  const size_t es = 2 * src->eng->elem_size();
  void* ss = nullptr;
  void* sd = nullptr;
  int st = cuda_status(cudaMallocAsync(&ss, src->eng->spectrum_elems() * es, s), "alloc");
  if (st != FHP_OK) return st;
  st = cuda_status(cudaMallocAsync(&sd, dst->eng->spectrum_elems() * es, s), "alloc");
  if (st == FHP_OK) st = src->eng->forward_spectrum(x_src, ss, s);
  if (st == FHP_OK) st = dst->eng->pad_spectrum(ss, a, sd, s);
  double pn = 1.0;
  for (int i = 0; i < a.dim; ++i) pn *= a.N[i];
  if (st == FHP_OK) st = dst->eng->inverse_spectrum(sd, x_dst, 1.0 / pn, s);
  if (sd) cudaFreeAsync(sd, s);
  if (ss) cudaFreeAsync(ss, s);
  return st;
}

// right-hand sides, CG from zero and A_H of the plan's coefficient (the
// driver of applications.py:58-86): the engine's fused call, or for mixed
// plans the refined solve between the FP64 right-hand side and energy
static int homogenize_once(fhp_plan_s& plan, int proj, double tol, int maxiter, void* b, void* x,
                           bool keep_x, double* AH_host, fhp::SolveResult& r, cudaStream_t s) {
  fhp::EngineBase& e = *plan.eng;
  if (!plan.lo) return e.homogenize(proj, tol, maxiter, b, x, keep_x, AH_host, r, s);
  int st = e.rhs_macro(proj, b, s);
  if (st == FHP_OK) st = cg_mixed(plan, proj, b, nullptr, tol, maxiter, x, r, 1, s);
  if (st == FHP_OK) st = e.energy(x, 1, AH_host, s);
  return st;
}

int fhp_homogenize_host(fhp_plan plan, int proj, int coef_kind, const double* coef_host,
                        double tol, int maxiter, double* AH_host, int* kit_host,
                        double* norm_res_host, void* x_host, void* stream) {
  if (!plan || !coef_host || !AH_host) return bad("plan, coef_host and AH_host are required");
  PlanStream ps(plan, as_stream(stream));
  cudaStream_t s = ps.get();
  fhp::EngineBase& e = *plan->eng;
  int st = fhp_set_coefficient(plan, coef_kind, coef_host, 0, s);
  if (st != FHP_OK) return st;
  const size_t bytes = (size_t)loads_all(e) * e.dv() * e.voxels() * e.elem_size();
  // the plan's persistent scratch: repeated calls allocate nothing
  void* b = e.scratch(fhp::SCR_HOST_B, bytes);
  void* x = e.scratch(fhp::SCR_HOST_X, bytes);
  st = (b && x) ? FHP_OK : FHP_OOM;
  fhp::SolveResult r;
  if (st == FHP_OK) st = homogenize_once(*plan, proj, tol, maxiter, b, x, x_host != nullptr,
                                         AH_host, r, s);
  if (st == FHP_OK && x_host)
    st = cuda_status(cudaMemcpyAsync(x_host, x, bytes, cudaMemcpyDeviceToHost, s), "copy");
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  const int L = loads_all(e);
  for (int l = 0; l < L && l < (int)r.kit.size(); ++l) {
    if (kit_host) kit_host[l] = r.kit[l];
    if (norm_res_host) norm_res_host[l] = r.norm_res[l];
  }
  return st;
}

int fhp_homogenize_host_many(fhp_plan plan, int proj, int coef_kind, int count,
                             const double* const* coef_host, double tol, int maxiter,
                             double* AH_host, int* kit_host, double* norm_res_host,
                             void* stream) {
  if (!plan || count < 0 || (count > 0 && (!coef_host || !AH_host)))
    return bad("plan, coef_host and AH_host are required");
  if (proj != 1 && proj != 2) return bad("proj must be 1 or 2");
  if (coef_kind < FHP_COEF_ISO || coef_kind > FHP_COEF_FULL) return bad("bad coefficient kind");
  for (int k = 0; k < count; ++k)
    if (!coef_host[k]) return bad("every coefficient is required");
  if (count == 0) return FHP_OK;
  PlanStream ps(plan, as_stream(stream));
  cudaStream_t s = ps.get();
  fhp::EngineBase& e = *plan->eng;
  const int dv = e.dv();
  const int c = coef_kind == FHP_COEF_ISO ? 1 : coef_kind == FHP_COEF_SYM ? dv * (dv + 1) / 2
                                                                          : dv * dv;
  const size_t ncoef = (size_t)e.instances() * c * e.coef_voxels() * sizeof(double);
  const size_t bytes = (size_t)loads_all(e) * dv * e.voxels() * e.elem_size();
  void* stage[2] = {e.scratch(fhp::SCR_COEF_STAGE, ncoef), e.scratch(fhp::SCR_COEF_STAGE2, ncoef)};
  void* b = e.scratch(fhp::SCR_HOST_B, bytes);
  void* x = e.scratch(fhp::SCR_HOST_X, bytes);
  if (!stage[0] || !stage[1] || !b || !x) return FHP_OOM;
  if (!plan->copy) {
    cudaError_t ce = cudaStreamCreateWithFlags(&plan->copy, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && ce == cudaSuccess; ++i) {
      ce = cudaEventCreateWithFlags(&plan->copied[i], cudaEventDisableTiming);
      if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&plan->freed[i], cudaEventDisableTiming);
    }
    if (ce != cudaSuccess) return cuda_status(ce, "upload stream");
  }
  cudaStream_t cp = plan->copy;
  const int L = loads_all(e);
  const int Lc = e.loads();
  // the upload of coefficient k + 1 (on the plan's upload stream, into the
  // other buffer) runs while problem k is solved; a buffer is reused once
  // its coefficient has been converted into the plan
  auto upload = [&](int k) -> int {
    const int i = k & 1;
    int st = cuda_status(cudaStreamWaitEvent(cp, plan->freed[i], 0), "wait");
    if (st == FHP_OK)
      st = cuda_status(cudaMemcpyAsync(stage[i], coef_host[k], ncoef, cudaMemcpyHostToDevice, cp),
                       "upload");
    if (st == FHP_OK) st = cuda_status(cudaEventRecord(plan->copied[i], cp), "record");
    return st;
  };
  // the buffers start free (events recorded on the solve stream)
  int st = cuda_status(cudaEventRecord(plan->freed[0], s), "record");
  if (st == FHP_OK) st = cuda_status(cudaEventRecord(plan->freed[1], s), "record");
  if (st == FHP_OK) st = upload(0);
  for (int k = 0; k < count && st == FHP_OK; ++k) {
    const int i = k & 1;
    st = cuda_status(cudaStreamWaitEvent(s, plan->copied[i], 0), "wait");
    if (st == FHP_OK)
      st = e.set_coefficient(coef_kind, static_cast<const double*>(stage[i]), true, s);
    if (st == FHP_OK && plan->lo)
      st = plan->lo->set_coefficient(coef_kind, static_cast<const double*>(stage[i]), true, s);
    if (st == FHP_OK) st = cuda_status(cudaEventRecord(plan->freed[i], s), "record");
    if (st == FHP_OK && k + 1 < count) st = upload(k + 1);
    fhp::SolveResult r;
    if (st == FHP_OK)
      st = homogenize_once(*plan, proj, tol, maxiter, b, x, false,
                           AH_host + (size_t)k * e.instances() * Lc * Lc, r, s);
    for (int l = 0; l < L && l < (int)r.kit.size(); ++l) {
      if (kit_host) kit_host[(size_t)k * L + l] = r.kit[l];
      if (norm_res_host) norm_res_host[(size_t)k * L + l] = r.norm_res[l];
    }
  }
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  (void)cudaStreamSynchronize(cp);
  return st;
}

int fhp_fft_plan_create(fhp_plan* out, int dim, const int* n, int ncomp, int precision) {
  if (!out) return bad("out is NULL");
  *out = nullptr;
  if (dim != 2 && dim != 3) return bad("dim must be 2 or 3");
  if (!n) return bad("n is required");
  if (ncomp < 1 || ncomp > 6) return bad("ncomp must be in 1..6");
  fhp::PlanConfig cfg;
  cfg.dim = dim;
  for (int i = 0; i < dim; ++i) {
    if (n[i] < 1 || n[i] > 4096) return bad("bad grid sizes");
    cfg.N[i] = n[i];
    cfg.band[i] = n[i];
    cfg.Y[i] = 1.0;
  }
  cfg.physics = -1;
  cfg.ncomp = ncomp;
  cfg.nloads = 1;
  int st = FHP_OK;
  std::unique_ptr<fhp::EngineBase> e;
  if (precision == FHP_F64) e = fhp::make_engine_f64(cfg, &st);
  else if (precision == FHP_F32) e = fhp::make_engine_f32(cfg, &st);
  else return bad("unknown precision");
  if (!e) return st == FHP_OK ? FHP_CUDA : st;
  auto* p = new (std::nothrow) fhp_plan_s;
  if (!p) return FHP_OOM;
  p->eng = std::move(e);
  *out = p;
  return FHP_OK;
}

int fhp_ga_grid_coefficient(fhp_plan plan_img, fhp_plan plan_out, const void* image,
                            const int* src_index, const double* weights, void* out,
                            void* stream) {
  if (!plan_img || !plan_out || !image || !src_index || !weights || !out)
    return bad("plans, image, tables and out are required");
  if (one_cell(plan_img) || one_cell(plan_out)) return FHP_BAD_ARG;
  const fhp::PlanConfig& a = plan_img->eng->config();
  const fhp::PlanConfig& b = plan_out->eng->config();
  if (a.dim != b.dim || plan_img->eng->dv() * plan_img->eng->loads() !=
                            plan_out->eng->dv() * plan_out->eng->loads() ||
      plan_img->eng->precision() != plan_out->eng->precision())
    return bad("plans differ in dim, field count or precision");
  cudaStream_t s = as_stream(stream);
  int nt = 0;
  for (int i = 0; i < b.dim; ++i) nt += b.N[i];
  // tables in the padded 3-axis order used by the kernels (n0 = 1 for 2D)
  std::vector<int> idx;
  std::vector<double> w;
  if (b.dim == 2) { idx.push_back(0); w.push_back(1.0); }
  idx.insert(idx.end(), src_index, src_index + nt);
  w.insert(w.end(), weights, weights + nt);
  for (int i = 0; i < b.dim; ++i) {
    int off = 0;
    for (int j = 0; j < i; ++j) off += b.N[j];
    for (int t = 0; t < b.N[i]; ++t) {
      const int v = src_index[off + t];
      if (v < 0 || v >= a.N[i]) return bad("source index out of range");
    }
  }
  const size_t es = 2 * plan_img->eng->elem_size();
  void *ss = nullptr, *sd = nullptr, *di = nullptr, *dw = nullptr;
  int st = cuda_status(cudaMallocAsync(&ss, plan_img->eng->spectrum_elems() * es, s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocAsync(&sd, plan_out->eng->spectrum_elems() * es, s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocAsync(&di, idx.size() * sizeof(int), s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocAsync(&dw, w.size() * sizeof(double), s), "alloc");
  if (st == FHP_OK)
    st = cuda_status(cudaMemcpyAsync(di, idx.data(), idx.size() * sizeof(int),
                                     cudaMemcpyHostToDevice, s), "copy");
  if (st == FHP_OK)
    st = cuda_status(cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(double),
                                     cudaMemcpyHostToDevice, s), "copy");
  if (st == FHP_OK) st = plan_img->eng->forward_spectrum(image, ss, s);
  if (st == FHP_OK)
    st = plan_out->eng->ga_gather(ss, a, static_cast<const int*>(di),
                                  static_cast<const double*>(dw), sd, s);
  if (st == FHP_OK) st = plan_out->eng->inverse_spectrum(sd, out, 1.0, s);
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  for (void* p : {ss, sd, di, dw})
    if (p) cudaFreeAsync(p, s);
  return st;
}

int fhp_ball_characteristic(fhp_plan plan, double r, double volume, const double* sq,
                            const double* phase, void* out, void* stream) {
  if (!plan || !sq || !phase || !out) return bad("plan, tables and out are required");
  if (one_cell(plan)) return FHP_BAD_ARG;
  if (!(r >= 0) || !(volume > 0)) return bad("r must be >= 0 and volume > 0");
  const fhp::PlanConfig& c = plan->eng->config();
  if (plan->eng->precision() != FHP_F64 || plan->eng->dv() * plan->eng->loads() != 1)
    return bad("the plan must be an FP64 FFT plan of one component");
  int g[3] = {1, 1, 1}, tot = 0;
  for (int i = 0; i < c.dim; ++i) {
    if (c.N[i] % 2 == 0) return bad("the grid must be odd on every axis");
    g[3 - c.dim + i] = c.N[i];
    tot += c.N[i];
  }
  // tables in the padded 3-axis order (a one-point axis 0 for 2D)
  std::vector<double> hs, hp;
  if (c.dim == 2) { hs.push_back(0.); hp.push_back(1.); hp.push_back(0.); }
  hs.insert(hs.end(), sq, sq + tot);
  hp.insert(hp.end(), phase, phase + 2 * tot);
  cudaStream_t s = as_stream(stream);
  void *dsq = nullptr, *dph = nullptr, *spec = nullptr;
  int st = cuda_status(cudaMallocAsync(&dsq, hs.size() * sizeof(double), s), "alloc");
  if (st == FHP_OK) st = cuda_status(cudaMallocAsync(&dph, hp.size() * sizeof(double), s), "alloc");
  if (st == FHP_OK)
    st = cuda_status(cudaMallocAsync(&spec, plan->eng->spectrum_elems() * 2 * sizeof(double), s),
                     "alloc");
  if (st == FHP_OK)
    st = cuda_status(cudaMemcpyAsync(dsq, hs.data(), hs.size() * sizeof(double),
                                     cudaMemcpyHostToDevice, s), "copy");
  if (st == FHP_OK)
    st = cuda_status(cudaMemcpyAsync(dph, hp.data(), hp.size() * sizeof(double),
                                     cudaMemcpyHostToDevice, s), "copy");
  if (st == FHP_OK)
    st = fhp::ball_spectrum(static_cast<const double*>(dsq), static_cast<const double*>(dph),
                            g[0], g[1], g[2], r, 1.0 / volume, spec, s);
  if (st == FHP_OK) st = plan->eng->inverse_spectrum(spec, out, 1.0, s);
  // the host tables are copied by the time the stream reaches this point
  if (st == FHP_OK) st = cuda_status(cudaStreamSynchronize(s), "sync");
  for (void* p : {dsq, dph, spec})
    if (p) cudaFreeAsync(p, s);
  return st;
}

int fhp_profile_enable(fhp_plan plan, int enable) {
  if (!plan) return bad("plan is NULL");
  for (fhp::EngineBase* e : {plan->eng.get(), plan->lo.get()}) {
    if (!e) continue;
    e->prof.reset();
    e->prof.on = enable != 0;
  }
  return FHP_OK;
}

int fhp_profile_read(fhp_plan plan, int max_kinds, char* names, long long* launches,
                     double* total_ms, double* bytes_per_launch, int* nkinds) {
  if (!plan || !nkinds) return bad("plan and nkinds are required");
  int k = 0;
  for (fhp::EngineBase* e : {plan->eng.get(), plan->lo.get()}) {
    if (!e) continue;
    e->prof.collect();
    for (const fhp::ProfEntry& p : e->prof.kinds) {
      if (k < max_kinds) {
        if (names) {
          std::strncpy(names + 64 * k, p.name.c_str(), 63);
          names[64 * k + 63] = 0;
        }
        if (launches) launches[k] = p.launches;
        if (total_ms) total_ms[k] = p.ms;
        if (bytes_per_launch) bytes_per_launch[k] = p.bytes;
      }
      ++k;
    }
  }
  *nkinds = k;
  return FHP_OK;
}

long long fhp_plan_launches(fhp_plan plan) {
  if (!plan) return 0;
  return plan->eng->launches + (plan->lo ? plan->lo->launches : 0);
}

}  // extern "C"
