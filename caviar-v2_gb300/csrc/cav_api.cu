// cav_api.cu -- the extern "C" boundary (include/cavgpu.h): context life cycle,
// uploads/downloads in the reference's host layouts, step orchestration with
// CUDA graphs, batches of replicas, and the parity exports.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

#include "cav_common.cuh"

using namespace cav;

namespace {

constexpr int MAX_GRAPH_STEPS = 1000;  // steps captured per graph, and thermo records per chunk

// A chunk of S steps launched as one unit (one captured graph, or directly).
// fuse[k]: step k's pair kernel also does step k + 1's drift (Fuse), so that a step is
// one launch; steps that begin a chunk, or follow a step that did not drift them,
// launch their drift kernel.  The fused steps of a chunk are made even in number,
// so that the gathered coordinates (FP64 positions or mixed rel), which alternate
// between two buffers at every fused step, end the chunk in the buffer they began.
struct ChunkPlan {
  int S = 0, ev = 0;          // steps; record period (thermo at step k iff ev > 0 and (k + 1) % ev == 0)
  std::vector<uint8_t> fuse;  // [S]
  bool thermo(int k) const { return ev > 0 && (k + 1) % ev == 0; }
  int fused_before(int k) const {
    int n = 0;
    for (int j = 0; j < k; ++j) n += fuse[j];
    return n;
  }
};

struct GraphEntry {
  int S, every, prof;
  cudaGraphExec_t exec;
  long long launches;  // kernels one replay launches outside the conditional rebuild bodies
  ChunkPlan plan;
};

// autotuner results, per process: a system of the same kind and size on the same
// device reuses the launch shape measured for the first one
struct TuneKey {
  int dev, precision, integrator, nrep, natoms, ntypes, force_kernel;
  bool operator==(const TuneKey &o) const {
    return dev == o.dev && precision == o.precision && integrator == o.integrator && nrep == o.nrep &&
           natoms == o.natoms && ntypes == o.ntypes && force_kernel == o.force_kernel;
  }
};
struct TuneChoice {
  int tpa, block, spg, seg;
};
std::mutex g_tune_mu;
std::vector<std::pair<TuneKey, TuneChoice>> g_tune_cache;

}  // namespace

struct cavgpu_ctx {
  cavgpu_params p{};
  Dev d{};
  Box b{};
  StepConsts sc{};
  LaunchCfg lc{};
  ThermoCfg tc{};
  PairTab tab_h{};
  std::vector<RepBox> reps;     // host copy of the replica boxes
  cudaStream_t st = nullptr;
  cudaStream_t side = nullptr;  // captures the bodies of the conditional rebuild nodes
  int natoms = 0;               // atoms over all replicas
  NveCfg nve{};                 // constraint::Nve (step 0 = off)
  bool uploaded = false, set_up = false;
  long long steps_done = 0;
  long long graph_launches = 0, kernel_launches = 0;
  int max_nb = 0;
  std::deque<GraphEntry> graphs;                      // stable references (chunks in flight hold them)
  std::map<std::pair<int, int>, ChunkPlan> eager_plans;  // chunks launched from the host
  // status words of the last chunks, read back without a full synchronisation
  int *h_status = nullptr;   // pinned, 2 x F_NWORDS
  cudaEvent_t ev_status[2] = {nullptr, nullptr};
  // reference binning (Neighborlist::init, src/neighborlist.cpp:334-342), single system
  double cutoff_extra = 0.0, cutoff_inv = 0.0, lo_local[3] = {0, 0, 0};
  int ref_nb[3] = {0, 0, 0};
  // profiling
  bool prof = false;
  std::vector<cudaEvent_t> ev0, ev1;
  double prof_ms = 0.0;
  long long prof_launches = 0;
  // allocations
  std::vector<void *> allocs;
  size_t nbr_bytes = 0;
};

namespace {

// name of the last CUDA error seen by this library (per thread, for diagnostics)
thread_local const char *g_last_cuda_error = "none";

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return CAVGPU_OK;
  g_last_cuda_error = cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? CAVGPU_E_NOMEM : CAVGPU_E_CUDA;
}

#define CK(x)                        \
  do {                               \
    int _rc = cuda_rc(x);            \
    if (_rc) return _rc;             \
  } while (0)
#define RK(x)              \
  do {                     \
    int _rc = (x);         \
    if (_rc) return _rc;   \
  } while (0)

template <class T>
int dalloc(cavgpu_ctx *c, T **p, size_t count) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) { cudaGetLastError(); return CAVGPU_E_NOMEM; }
  c->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return CAVGPU_OK;
}

void free_graphs(cavgpu_ctx *c) {
  for (auto &g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
}

bool is_lang(const cavgpu_ctx *c) { return c->p.integrator == CAVGPU_VELOCITY_VERLET_LANGEVIN; }

// thermo folds after the force kernel of a thermo step
int enqueue_thermo_after_force(cavgpu_ctx *c, int ring_slot, long long *nl) {
  const bool lang = is_lang(c);
  if (c->b.nrep == 1) {
    const int nb_ke = lang ? drift_grid_blocks(c->lc) : force_grid_blocks(c->lc);
    RK(launch_thermo_final(c->d, c->tc, nb_ke, force_grid_blocks(c->lc), lang ? force_grid_blocks(c->lc) : 0,
                           ring_slot, c->st));
  } else {
    RK(launch_thermo_replicas(c->d, c->b, c->tc, lang ? 0 : 1, 1, c->st));
  }
  *nl += 1;
  return CAVGPU_OK;
}

// drift (VV) or first Langevin half; batches fold their per-replica KE right after
// the Langevin half kick, where the reference takes the temperature.  Langevin
// with constraint::Nve: the velocity half, Nve on the mid-step velocities
// (src/md_simulator.cpp:782-793), then the temperature and the position update.
// `view` holds the buffers current at this step.
int enqueue_drift(cavgpu_ctx *c, const Dev &view, int k, bool thermo, long long *nl) {
  if (is_lang(c) && c->nve.step > 0) {
    RK(launch_drift(view, c->b, c->sc, c->lc, k, -1, c->st));
    RK(launch_nve(view, c->b, c->tc, c->nve, k, 0, -1, c->st));
    RK(launch_lang_pos(view, c->b, c->sc, c->lc, thermo ? 1 : 0, c->st));
    *nl += 5;
    return CAVGPU_OK;
  }
  RK(launch_drift(view, c->b, c->sc, c->lc, k, thermo && is_lang(c), c->st));
  *nl += 1;
  if (thermo && is_lang(c) && c->b.nrep > 1) {
    RK(launch_thermo_replicas(view, c->b, c->tc, 1, 0, c->st));
    *nl += 1;
  }
  return CAVGPU_OK;
}

int fuse_mode(const cavgpu_ctx *c) {
  if (c->p.integrator == CAVGPU_VELOCITY_VERLET) return FUSE_VV;
  if (c->p.integrator == CAVGPU_LEAP_FROG) return FUSE_LF;
  return FUSE_LANG;
}

// Which steps of a chunk drift the next one.  Not with constraint::Nve (it rescales
// the velocities between the kick and the next drift); Langevin: not into a step
// whose temperature is recorded (the mid-step sums come from the drift kernel);
// leap-frog: not out of a recorded step (the closing velocities are read after it).
ChunkPlan make_plan(const cavgpu_ctx *c, int S, int ev) {
  ChunkPlan pl;
  pl.S = S;
  pl.ev = ev;
  pl.fuse.assign(S, 0);
  if (c->nve.step > 0) return pl;
  int nf = 0, last = -1;
  for (int k = 0; k + 1 < S; ++k) {
    if (is_lang(c) && pl.thermo(k + 1)) continue;
    if (c->p.integrator == CAVGPU_LEAP_FROG && pl.thermo(k)) continue;
    pl.fuse[k] = 1;
    ++nf;
    last = k;
  }
  if (nf & 1) pl.fuse[last] = 0;  // an even number: the buffers end where they began
  return pl;
}

// The steps of a chunk, captured into the graph being recorded on c->st (capture)
// or launched directly.  A step: [drift kernel] -> rebuild kernels, behind a
// conditional node in a graph (they return at once without a half-skin trigger when
// launched directly) -> pair kernel with the closing update [and the next drift]
// [and, single systems, the thermo fold in its last block] -> [thermo fold kernel:
// batches, constraint::Nve] -> [constraint::Nve].  The conditional value comes from the
// condition kernel after a drift kernel, else from the previous pair kernel.
int enqueue_chunk(cavgpu_ctx *c, const ChunkPlan &pl, bool capture, long long *launches) {
  Dev view = c->d;
  const bool mixed = c->p.precision == CAVGPU_MIXED;
  long long nl = 0;
  cudaGraphConditionalHandle hnext = 0;
  for (int k = 0; k < pl.S; ++k) {
    const bool th = pl.thermo(k);
    const int ring_slot = th ? (k + 1) / pl.ev - 1 : -1;
    const bool separate = k == 0 || !pl.fuse[k - 1];
    if (separate) RK(enqueue_drift(c, view, k, th, &nl));
    if (capture) {
      cudaStreamCaptureStatus cs;
      cudaGraph_t g = nullptr;
      CK(cudaStreamGetCaptureInfo(c->st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
      cudaGraphConditionalHandle h = hnext;
      if (separate) {
        CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        RK(launch_set_rebuild_cond(view, h, c->st));
        nl += 1;
      }
      const cudaGraphNode_t *deps = nullptr;
      size_t nd = 0;
      CK(cudaStreamGetCaptureInfo(c->st, &cs, nullptr, &g, &deps, nullptr, &nd));
      // the params struct holds a union without a default constructor: zeroed storage
      alignas(cudaGraphNodeParams) unsigned char cp_raw[sizeof(cudaGraphNodeParams)];
      std::memset(cp_raw, 0, sizeof(cp_raw));
      cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_raw);
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t cond = nullptr;
      CK(cudaGraphAddNode(&cond, g, deps, nullptr, nd, &cp));
      CK(cudaStreamBeginCaptureToGraph(c->side, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal));
      const int brc = launch_rebuild(view, c->b, c->lc, 0, c->side);
      cudaGraph_t body = nullptr;
      const cudaError_t be = cudaStreamEndCapture(c->side, &body);
      RK(brc);
      CK(be);
      CK(cudaStreamUpdateCaptureDependencies(c->st, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
    } else {
      if (separate) {
        RK(launch_halt_check(view, c->st));
        nl += 1;
      }
      RK(launch_rebuild(view, c->b, c->lc, 0, c->st));
      nl += rebuild_kernels(c->b);
    }
    const int fuse = pl.fuse[k] ? fuse_mode(c) : FUSE_NONE;
    int set_cond = 0;
    hnext = 0;
    if (fuse && capture) {
      cudaStreamCaptureStatus cs;
      cudaGraph_t g = nullptr;
      CK(cudaStreamGetCaptureInfo(c->st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
      CK(cudaGraphConditionalHandleCreate(&hnext, g, 0, cudaGraphCondAssignDefault));
      set_cond = 1;
    }
    if (c->prof && k < (int)c->ev0.size())
      CK(capture ? cudaEventRecordWithFlags(c->ev0[k], c->st, cudaEventRecordExternal) : cudaEventRecord(c->ev0[k], c->st));
    // a recorded step of a single system: the pair kernel's last block folds the record
    const bool fold = th && c->b.nrep == 1 && c->nve.step == 0;
    FoldArgs fa{c->tc, is_lang(c) ? drift_grid_blocks(c->lc) : force_grid_blocks(c->lc),
                is_lang(c) ? force_grid_blocks(c->lc) : 0, ring_slot};
    RK(launch_force(view, c->b, c->sc, c->lc, is_lang(c) ? 2 : 1, th, k, fuse, set_cond, hnext, c->st,
                    fold ? &fa : nullptr));
    if (c->prof && k < (int)c->ev1.size())
      CK(capture ? cudaEventRecordWithFlags(c->ev1[k], c->st, cudaEventRecordExternal) : cudaEventRecord(c->ev1[k], c->st));
    nl += 1;
    if (fuse) {  // the next step gathers the coordinates this launch wrote
      if (mixed) std::swap(view.rel, view.rel_alt);
      else std::swap(view.pos, view.pos_alt);
    }
    if (th && !fold) RK(enqueue_thermo_after_force(c, ring_slot, &nl));
    if (c->nve.step > 0 && !is_lang(c)) {  // constraint::Nve after the temperature (src/md_simulator.cpp:681-694)
      RK(launch_nve(view, c->b, c->tc, c->nve, k, th, ring_slot, c->st));
      nl += 3;
    }
  }
  RK(launch_advance_step(view, c->st));
  *launches = nl + 1;
  return CAVGPU_OK;
}

int ensure_events(cavgpu_ctx *c, int S) {
  while ((int)c->ev0.size() < S) {
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    c->ev0.push_back(a);
    c->ev1.push_back(b);
  }
  return CAVGPU_OK;
}

int collect_profile(cavgpu_ctx *c, int count) {
  CK(cudaStreamSynchronize(c->st));
  for (int k = 0; k < count; ++k) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0[k], c->ev1[k]));
    c->prof_ms += ms;
    c->prof_launches += 1;
  }
  return CAVGPU_OK;
}

GraphEntry *get_graph(cavgpu_ctx *c, int S, int every, int *rc) {
  for (auto &g : c->graphs)
    if (g.S == S && g.every == every && g.prof == (int)c->prof) return &g;
  *rc = CAVGPU_OK;
  if (c->prof && (*rc = ensure_events(c, S))) return nullptr;
  GraphEntry ge{S, every, (int)c->prof, nullptr, 0, make_plan(c, S, every)};
  cudaGraph_t graph = nullptr;
  if ((*rc = cuda_rc(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal)))) return nullptr;
  const int erc = enqueue_chunk(c, ge.plan, true, &ge.launches);
  cudaError_t e = cudaStreamEndCapture(c->st, &graph);
  if (erc || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    *rc = erc ? erc : CAVGPU_E_CUDA;
    return nullptr;
  }
  e = cudaGraphInstantiate(&ge.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) { *rc = CAVGPU_E_CUDA; return nullptr; }
  c->graphs.push_back(std::move(ge));
  return &c->graphs.back();
}

int read_flags(cavgpu_ctx *c, int *f) {
  CK(cudaMemcpyAsync(f, c->d.flags, F_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return CAVGPU_OK;
}

int check_status(cavgpu_ctx *c) {
  int f[F_NWORDS];
  RK(read_flags(c, f));
  c->max_nb = std::max(c->max_nb, f[F_MAXNB]);
  if (f[F_NAN]) return CAVGPU_E_NAN;
  if (f[F_OVERFLOW]) return CAVGPU_E_NLIST_OVERFLOW;
  return CAVGPU_OK;
}

// (re)allocate the neighbour list for `cap` slots per atom
int alloc_nbr(cavgpu_ctx *c, int cap) {
  cap = (cap + 63) / 64 * 64;  // nbr_index needs cap % (4 * tpa) == 0, tpa <= 16
  const int A = 32 / c->d.tpa;  // whole blocks of A slots (nbr_index)
  const size_t bytes = (size_t)((c->b.nslot + A - 1) / A) * A * (size_t)cap * sizeof(uint32_t);
  if (c->d.nbr) {
    auto it = std::find(c->allocs.begin(), c->allocs.end(), (void *)c->d.nbr);
    if (it != c->allocs.end()) c->allocs.erase(it);
    cudaFree(c->d.nbr);
    c->d.nbr = nullptr;
  }
  void *q = nullptr;
  if (cudaMalloc(&q, bytes) != cudaSuccess) { cudaGetLastError(); return CAVGPU_E_NOMEM; }
  c->allocs.push_back(q);
  c->d.nbr = static_cast<uint32_t *>(q);
  c->d.cap = cap;
  c->nbr_bytes = bytes;
  free_graphs(c);  // graphs hold the old Dev by value
  return CAVGPU_OK;
}

// forced list build of every replica; grows the capacity until the build fits.
// Clears every status word but the rebuild counts; with count = false those stay
// as they were (a build that completes a step whose own rebuild overflowed, or
// that restarts from a snapshot, is not a rebuild of the trajectory).
int forced_build(cavgpu_ctx *c, bool count = true) {
  int f0[F_NWORDS];
  RK(read_flags(c, f0));
  for (int attempt = 0; attempt < 4; ++attempt) {
    int zero[F_NWORDS] = {0};
    int f[F_NWORDS];
    if (attempt == 0) std::memcpy(f, f0, sizeof(f));  // nothing ran since f0 was read
    else RK(read_flags(c, f));
    zero[F_REBUILDS] = f[F_REBUILDS];
    zero[F_PASSES] = f[F_PASSES];
    CK(cudaMemcpyAsync(c->d.flags, zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
    RK(launch_rebuild(c->d, c->b, c->lc, 1, c->st));
    c->kernel_launches += rebuild_kernels(c->b);
    RK(read_flags(c, f));
    c->max_nb = f[F_MAXNB];
    if (!f[F_OVERFLOW]) {
      if (!count) {
        f[F_REBUILDS] = f0[F_REBUILDS];
        f[F_PASSES] = f0[F_PASSES];
        CK(cudaMemcpyAsync(c->d.flags, f, sizeof(f), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
      }
      return CAVGPU_OK;
    }
    RK(alloc_nbr(c, (int)(f[F_OVERFLOW] * 1.25) + 32));
  }
  return CAVGPU_E_NLIST_OVERFLOW;
}

// box and search grid of one replica; L >= 2 cutoff_extra (one image per pair)
int make_repbox(double ce, const double lo[3], const double hi[3], RepBox *rb) {
  for (int a = 0; a < 3; ++a) {
    rb->lo[a] = lo[a];
    rb->hi[a] = hi[a];
    rb->L[a] = hi[a] - lo[a];  // Domain::update_after_domain_change (src/domain.cpp:498)
    if (!(rb->L[a] >= 2.0 * ce)) return CAVGPU_E_ARG;
    int nc = (int)std::floor(rb->L[a] / ce);
    while (nc > 1 && rb->L[a] / nc < ce * (1.0 + 1e-10)) --nc;  // cell width safely >= ce
    rb->nc[a] = std::max(nc, 1);
    rb->w[a] = rb->L[a] / rb->nc[a];
    rb->inv_w[a] = 1.0 / rb->w[a];
    rb->wf[a] = (float)rb->w[a];
    rb->wlo[a] = (float)(rb->w[a] - (double)rb->wf[a]);
  }
  rb->ncell = rb->nc[0] * rb->nc[1] * rb->nc[2];
  return CAVGPU_OK;
}

int create_common(const cavgpu_params *p, int nrep, const double *lo3, const double *hi3, cavgpu_ctx **out) {
  if (!p || !out || nrep < 1 || !lo3 || !hi3) return CAVGPU_E_ARG;
  *out = nullptr;
  if (p->ntypes < 1 || p->ntypes > CAVGPU_MAX_TYPES) return CAVGPU_E_ARG;
  if (p->bc[0] != 1 || p->bc[1] != 1 || p->bc[2] != 1) return CAVGPU_E_ARG;
  if (!(p->nl_cutoff > 0.0) || !(p->nl_coef >= 1.0) || !(p->lj_cutoff >= 0.0) || !(p->dt >= 0.0)) return CAVGPU_E_ARG;
  if (p->precision != CAVGPU_FP64 && p->precision != CAVGPU_MIXED) return CAVGPU_E_ARG;
  if (p->integrator != CAVGPU_VELOCITY_VERLET && p->integrator != CAVGPU_VELOCITY_VERLET_LANGEVIN &&
      p->integrator != CAVGPU_LEAP_FROG)
    return CAVGPU_E_ARG;
  if (p->n_r_df < 0 || p->n_r_df > 3) return CAVGPU_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) { cudaGetLastError(); return CAVGPU_E_CUDA; }
  cavgpu_ctx *c = new (std::nothrow) cavgpu_ctx();
  if (!c) return CAVGPU_E_NOMEM;
  c->p = *p;
  const double ce = p->nl_cutoff * p->nl_coef;  // Neighborlist::init (src/neighborlist.cpp:317)
  c->cutoff_extra = ce;
  c->reps.resize(nrep);
  for (int r = 0; r < nrep; ++r)
    if (make_repbox(ce, lo3 + 3 * r, hi3 + 3 * r, &c->reps[r])) { delete c; return CAVGPU_E_ARG; }
  // reference binning of a single system: Domain::calculate_local_domain with grid
  // index 0 of 1 (src/domain.cpp:320-326), no_bins = ceil(size * 1/cutoff_extra)
  c->cutoff_inv = 1.0 / ce;
  for (int a = 0; a < 3; ++a) {
    c->lo_local[a] = lo3[a] + (hi3[a] - lo3[a]) * 0 / 1;
    const double hi_local = lo3[a] + (hi3[a] - lo3[a]) * 1 / 1;
    c->ref_nb[a] = (int)std::ceil((hi_local - c->lo_local[a]) * c->cutoff_inv);
  }
  Box &b = c->b;
  b.nrep = nrep;
  b.ce2 = ce * ce;
  b.ce2_lo = (float)(b.ce2 * (1.0 - 2e-4));
  b.ce2_hi = (float)(b.ce2 * (1.0 + 2e-4));
  b.thr2 = 0.25 * (ce - p->nl_cutoff) * (ce - p->nl_cutoff);
  b.thr2f = (float)(b.thr2 * (1.0 - 1e-6));
  // pair table (force_field::Lj, src/force/lj.cpp:453-484)
  PairTab &t = c->tab_h;
  const int nt = p->ntypes;
  t.nt = nt;
  for (int a = 0; a < nt; ++a)
    for (int q = 0; q < nt; ++q) {
      const int k = a * nt + q;
      const double rc = p->cutoff_list_on ? p->cutoff_list[k] : p->lj_cutoff;
      const double rc2 = rc * rc, eps = p->eps[k], sig = p->sigma[k];
      if (rc < 0.0) { delete c; return CAVGPU_E_ARG; }
      t.rc2[k] = eps == 0.0 ? -1.0 : rc2;
      t.sig2[k] = sig * sig;
      t.eps4[k] = 4.0 * eps;
      const double sc2 = rc2 > 0 ? sig * sig / rc2 : 0.0, sc6 = sc2 * sc2 * sc2;
      t.gc[k] = rc2 > 0 ? 4.0 * eps * sc6 * (6.0 - 12.0 * sc6) / rc2 : 0.0;
      t.uc[k] = 4.0 * eps * (sc6 * sc6 - sc6);
    }
  for (int a = 0; a < nt; ++a) {
    t.mass[a] = p->mass[a];
    t.minv[a] = p->mass[a] == 0.0 ? 0.0 : 1.0 / p->mass[a];  // Atom_data::add_type_mass (src/atom_data.cpp:368-383)
  }
  // integrator constants (src/md_simulator.cpp:394-405)
  StepConsts &sc = c->sc;
  sc.dt = p->dt;
  sc.hdt = 0.5 * p->dt;
  sc.hdt2 = 0.5 * p->dt * p->dt;
  if (p->integrator == CAVGPU_VELOCITY_VERLET_LANGEVIN) {
    const double fr = p->lang_friction, dt = p->dt;
    sc.la = (2.0 - fr * dt) / (2.0 + fr * dt);
    if (p->lang_kbt > 0) sc.lb = std::sqrt(p->lang_kbt * fr * 0.5 * dt);
    else if (p->lang_kb > 0 && p->lang_temperature > 0) sc.lb = std::sqrt(p->lang_kb * p->lang_temperature * fr * 0.5 * dt);
    else { delete c; return CAVGPU_E_ARG; }
    sc.lc = 2.0 * dt / (2.0 + fr * dt);
  }
  sc.seed = p->seed;
  sc.noise_off = p->noise_off;
  if (p->jump_tol < 0.0 || p->initial_step < 0) { delete c; return CAVGPU_E_ARG; }
  if (p->nve_step > 0) {  // constraint::Nve: one system (checked at upload)
    if (p->nve_mode < CAVGPU_NVE_ENERGY_PER_DOF || p->nve_mode > CAVGPU_NVE_KB_TEMPERATURE || !(p->nve_value > 0.0) ||
        (p->nve_mode == CAVGPU_NVE_KB_TEMPERATURE && !(p->nve_kb > 0.0))) {
      delete c;
      return CAVGPU_E_ARG;
    }
    c->nve.step = p->nve_step;
    c->nve.mode = p->nve_mode;
    c->nve.value = p->nve_value;
    c->nve.kb = p->nve_kb;
  }
  sc.jump_tol = p->jump_tol;  // Lj::set_jump_tol (src/force/lj.cpp:82-86); 0 = off
  sc.jump_tolf = (float)p->jump_tol;
  // launch shape
  c->lc.precision = p->precision;
  c->lc.integrator = p->integrator;
  c->lc.tpa = p->threads_per_atom ? p->threads_per_atom : 4;
  c->lc.block = p->block_size ? p->block_size : 128;
  if (c->lc.tpa != 1 && c->lc.tpa != 2 && c->lc.tpa != 4 && c->lc.tpa != 8 && c->lc.tpa != 16) { delete c; return CAVGPU_E_ARG; }
  if (c->lc.block < 32 || c->lc.block > 256 || c->lc.block % 32) { delete c; return CAVGPU_E_ARG; }
  if (p->force_kernel < CAVGPU_FORCE_AUTO || p->force_kernel > CAVGPU_FORCE_SEGMENTS) { delete c; return CAVGPU_E_ARG; }
  c->lc.use_seg = p->precision == CAVGPU_MIXED && p->force_kernel == CAVGPU_FORCE_SEGMENTS;
  c->lc.ntypes = p->ntypes;
  c->d.tpa = c->lc.tpa;
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) { delete c; return CAVGPU_E_CUDA; }
  if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(c->st);
    delete c;
    return CAVGPU_E_CUDA;
  }
  int rc = dalloc(c, &c->d.tab, 1);
  if (!rc) rc = dalloc(c, &c->d.flags, F_NWORDS);
  if (!rc) rc = dalloc(c, &c->d.thermo, 8);
  if (!rc) rc = dalloc(c, &c->d.step_base, 1);
  if (!rc) rc = dalloc(c, &c->d.thermo_ring, THERMO_REC * (size_t)MAX_GRAPH_STEPS);
  if (!rc) rc = dalloc(c, &c->d.fold, 10 * (size_t)THERMO_FOLD_BLOCKS);
  if (!rc) rc = dalloc(c, &c->d.scan_part, (size_t)SCAN_SLICES);
  if (!rc) rc = dalloc(c, &c->d.fold_ticket, 1);
  if (!rc) rc = cuda_rc(cudaMemsetAsync(c->d.fold_ticket, 0, sizeof(unsigned int), c->st));
  if (!rc) rc = dalloc(c, &c->d.force_ticket, 1);
  if (!rc) rc = cuda_rc(cudaMemsetAsync(c->d.force_ticket, 0, sizeof(unsigned int), c->st));
  if (!rc) rc = cuda_rc(cudaMemcpyAsync(c->d.tab, &c->tab_h, sizeof(PairTab), cudaMemcpyHostToDevice, c->st));
  if (!rc) rc = cuda_rc(cudaMemsetAsync(c->d.flags, 0, F_NWORDS * sizeof(int), c->st));
  if (!rc) rc = cuda_rc(cudaMemsetAsync(c->d.thermo, 0, 8 * sizeof(double), c->st));
  const long long step0 = p->initial_step;  // Md_simulator::initial_step
  if (!rc) rc = cuda_rc(cudaMemcpyAsync(c->d.step_base, &step0, sizeof(long long), cudaMemcpyHostToDevice, c->st));
  if (!rc) rc = cuda_rc(cudaStreamSynchronize(c->st));
  if (rc) { cavgpu_destroy(c); return rc; }
  *out = c;
  return CAVGPU_OK;
}

// Row segments of the mixed force kernel.  Replica r's x-rows are cut into
// segments of S cells, S chosen so that the 9 x (S + 2) staged cells hold about
// STAGE_TARGET atoms at the replica's mean cell occupancy; the stage is sized
// for the largest estimate with 35% headroom (a segment that still overflows it
// falls back to global gathers).
int build_segments(cavgpu_ctx *c) {
  constexpr double STAGE_TARGET = 4096.0;
  constexpr int SEG_MAX = 62;  // cells per segment
  std::vector<int4> segs;
  int umax = 3;
  double need = 0.0;
  for (int r = 0; r < c->b.nrep; ++r) {
    const RepBox &rb = c->reps[r];
    if (rb.nc[1] > 0xffff || rb.nc[2] > 0x7fff) return CAVGPU_E_RANGE;
    const double navg = (double)rb.natoms / rb.ncell;
    const int smax = std::max(1, std::min(SEG_MAX, (int)(STAGE_TARGET / (9.0 * navg * 1.3)) - 2));
    const int ncx = rb.nc[0], nsx = (ncx + smax - 1) / smax, S = (ncx + nsx - 1) / nsx;
    for (int cz = 0; cz < rb.nc[2]; ++cz)
      for (int cy = 0; cy < rb.nc[1]; ++cy)
        for (int x0 = 0; x0 < ncx; x0 += S) segs.push_back(make_int4(r, cy | (cz << 16), x0, std::min(S, ncx - x0)));
    umax = std::max(umax, S + 2);
    need = std::max(need, 9.0 * (S + 2) * navg * 1.35);
  }
  // dynamic shared memory within the 227 KiB a block may hold, beside ~4 KiB of static
  const size_t limit = 227 * 1024 - 4096 - (size_t)2 * 9 * umax * sizeof(int);
  c->d.stage_cap = (int)std::min<double>(need + 128.0, (double)(limit / 16));
  int4 *dseg = nullptr;
  RK(dalloc(c, &dseg, segs.size()));
  CK(cudaMemcpyAsync(dseg, segs.data(), segs.size() * sizeof(int4), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->d.seg = dseg;
  c->d.nseg = (int)segs.size();
  c->d.seg_umax = umax;
  c->lc.nseg = c->d.nseg;
  return prepare_force_seg(seg_smem_bytes(c->d.stage_cap, umax));
}

// Lay the replicas out (32-aligned slot ranges, consecutive cell ranges with one
// padding cell each), allocate every per-slot array and upload the atoms.
int upload_common(cavgpu_ctx *c, const int64_t *counts, const double *pos3, const double *vel3,
                  const uint64_t *type, const uint64_t *id) {
  if (c->uploaded) return CAVGPU_E_STATE;
  const int R = c->b.nrep;
  int64_t total = 0, nslot = 0, ncell_all = 0;
  for (int r = 0; r < R; ++r) {
    if (counts[r] < 1) return CAVGPU_E_ARG;
    total += counts[r];
  }
  if (!pos3 || !type || total > MAX_ATOMS) return total > MAX_ATOMS ? CAVGPU_E_RANGE : CAVGPU_E_ARG;
  for (int r = 0; r < R; ++r) {
    RepBox &rb = c->reps[r];
    rb.slot_off = (int)nslot;
    rb.natoms = (int)counts[r];
    const int64_t end = nslot + counts[r];
    const int64_t next = R == 1 ? end : (end + SLOT_ALIGN - 1) / SLOT_ALIGN * SLOT_ALIGN;
    rb.pad = (int)(next - end);
    nslot = next;
    rb.cell_off = (int)ncell_all;
    ncell_all += rb.ncell + 1;
  }
  if (nslot > MAX_ATOMS || ncell_all > (1ll << 30)) return CAVGPU_E_RANGE;
  const int N = (int)total, NS = (int)nslot;
  // a single system goes to the device as the caller's arrays are and is converted
  // and checked there (k_upload_single); batches are laid out here
  const bool on_device = R == 1;
  std::vector<dbl4> hp, hv;
  std::vector<int> ht, rep_of, cell_rep;
  std::vector<uint32_t> hid;
  std::vector<char> seen;
  // atoms per type and replica: the total mass is sum_t mass_t n_t, in type order (exact
  // counts, the same value however the atoms are ordered or counted)
  std::vector<int64_t> ntype((size_t)R * CAVGPU_MAX_TYPES, 0);
  c->reps[0].id_off = 0;
  int64_t h = 0;
  if (!on_device) {
    hp.assign(NS, make_dbl4(0, 0, 0, 0));
    hv.assign(NS, make_dbl4(0, 0, 0, 0));
    ht.assign(NS, 0);
    rep_of.assign(NS, -1);
    cell_rep.assign(ncell_all, -1);
    hid.assign(NS, 0);
    seen.assign(id ? N : 0, 0);
  }
  for (int r = 0; r < R && !on_device; ++r) {
    RepBox &rb = c->reps[r];
    rb.id_off = (int)h;
    for (int k = 0; k < rb.natoms; ++k, ++h) {
      const int s = rb.slot_off + k;
      for (int a = 0; a < 3; ++a) {
        const double x = pos3[3 * h + a];
        // Atom_data::position_inside_global_domain (src/atom_data.cpp:548-559)
        if (!(x >= rb.lo[a] && x < rb.hi[a])) return CAVGPU_E_ARG;
      }
      if (type[h] >= (uint64_t)c->p.ntypes) return CAVGPU_E_ARG;
      const uint64_t ii = id ? id[h] : (uint64_t)k;  // batches: ids local to the replica
      if (ii >= (uint64_t)N || (id && seen[ii]++)) return CAVGPU_E_ARG;  // ids: a permutation of 0..n-1
      hp[s] = make_dbl4(pos3[3 * h], pos3[3 * h + 1], pos3[3 * h + 2], type_bits((int)type[h]));
      if (vel3) hv[s] = make_dbl4(vel3[3 * h], vel3[3 * h + 1], vel3[3 * h + 2], 0.0);
      ht[s] = (int)type[h];
      hid[s] = (uint32_t)ii;
      rep_of[s] = r;
      ++ntype[(size_t)r * CAVGPU_MAX_TYPES + type[h]];
    }
    for (int k = 0; k < rb.ncell; ++k) cell_rep[rb.cell_off + k] = r;
  }
  Box &b = c->b;
  b.nslot = NS;
  b.ncell_all = (int)ncell_all;
  b.r0 = c->reps[0];
  c->natoms = N;
  c->sc.n = NS;
  c->lc.n = NS;
  c->tc.n = N;
  c->tc.n_r_df = c->p.n_r_df;
  c->tc.k_b = c->p.k_b;
  // finalize_pressure_mpi_domain volume (src/atom_data/kinetic_energy.cpp:242-243) of the
  // single system: local domain of grid index 0 of 1; replicas use their box volume
  double vol = 1.0;
  for (int a = 0; a < 3; ++a) vol *= (c->reps[0].lo[a] + c->reps[0].L[a] * 1 / 1) - c->lo_local[a];
  c->tc.volume = vol;
  c->tc.langevin = is_lang(c);
  Dev &d = c->d;
  if (c->p.precision == CAVGPU_MIXED) RK(build_segments(c));
  // partial sums for the largest force grid of any launch shape and kernel (the
  // autotuner changes them later) and for the drift grid
  size_t nblk = 1;
  for (int seg = 0; seg < 2; ++seg)
    for (int tpa = 1; tpa <= 16; tpa *= 2)
      for (int blk = 32; blk <= 256; blk += 32) {
        LaunchCfg t = c->lc;
        t.tpa = tpa;
        t.block = blk;
        t.use_seg = seg;
        nblk = std::max(nblk, (size_t)force_grid_blocks(t));
      }
  const size_t nblk_d = (size_t)std::max((NS + 255) / 256, 1);
  d.partials_blocks = (int)nblk;
  int rc = CAVGPU_OK;
  // the per-slot and per-cell arrays, carved out of one allocation (one cudaMalloc
  // rather than thirty: part of the set-up cost a short run pays)
  {
    size_t total_bytes = 0;
    std::vector<std::pair<void **, size_t>> parts;
    auto take = [&](auto **p, size_t count) {
      using E = typename std::remove_pointer<typename std::remove_reference<decltype(*p)>::type>::type;
      parts.push_back({reinterpret_cast<void **>(p), total_bytes});
      total_bytes += (std::max<size_t>(count, 1) * sizeof(E) + 255) & ~(size_t)255;
    };
    for (dbl4 **pp : {&d.pos, &d.vel, &d.acc, &d.pos_ref, &d.t_pos, &d.t_vel, &d.t_acc}) take(pp, NS);
    take(&d.rel, NS);
    take(&d.rel_ref, NS);
    // the second buffer of the coordinates a pair kernel gathers (it drifts into it)
    if (c->p.precision == CAVGPU_MIXED) take(&d.rel_alt, NS);
    else take(&d.pos_alt, NS);
    for (int **pp : {&d.type, &d.cell_of, &d.t_type, &d.atom_cell, &d.perm, &d.perm_tmp, &d.nnbr}) take(pp, NS);
    take(&d.id, NS);
    take(&d.t_id, NS);
    take(&d.skey, NS);
    take(&d.cell_count, ncell_all);
    take(&d.cell_cursor, ncell_all);
    take(&d.cell_start, (size_t)ncell_all + 1);
    take(&d.partials_ke, 4 * std::max(nblk, nblk_d));
    take(&d.partials_ke_end, 4 * nblk);
    take(&d.partials_ev, 2 * nblk);
    take(&d.h3, 3 * (size_t)N);
    take(&d.hi3, 3 * (size_t)N);
    if (c->p.msd_process) {  // Atom_data::msd_process: boundary crossings per atom
      take(&d.img, NS);
      take(&d.t_img, NS);
    }
    if (c->p.ignore_intra_molecule) {
      take(&d.mol, NS);
      take(&d.t_mol, NS);
    }
    char *arena = nullptr;
    rc = dalloc(c, &arena, total_bytes);
    if (rc) return rc;
    for (auto &pt : parts) *pt.first = arena + pt.second;
  }
  if (c->p.msd_process) rc = cuda_rc(cudaMemsetAsync(d.img, 0, NS * sizeof(int4), c->st));  // zero at upload
  // molecule index -1 for every atom (Atom_data::add_atom) until set
  if (!rc && c->p.ignore_intra_molecule) rc = cuda_rc(cudaMemsetAsync(d.mol, 0xff, NS * sizeof(int), c->st));
  if (c->nve.step > 0) {
    if (R > 1) return CAVGPU_E_ARG;  // constraint::Nve acts on one system's kinetic energy
    if (!rc) rc = dalloc(c, &d.nve_partials, 4 * (size_t)NVE_BLOCKS);
    if (!rc) rc = dalloc(c, &d.nve_lambda, 1);
  }
  RepBox *drep = nullptr;
  int *dflag = nullptr;
  if (!rc) rc = dalloc(c, &drep, R);
  if (!rc) rc = dalloc(c, &dflag, R);
  if (R > 1) {
    int *drep_of = nullptr, *dcell_rep = nullptr;
    if (!rc) rc = dalloc(c, &drep_of, NS);
    if (!rc) rc = dalloc(c, &dcell_rep, ncell_all);
    if (!rc) rc = dalloc(c, &d.ev_atom, NS);
    if (!rc) rc = dalloc(c, &d.thermo_rep, 8 * (size_t)R);
    if (rc) return rc;
    CK(cudaMemcpyAsync(drep_of, rep_of.data(), NS * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(dcell_rep, cell_rep.data(), ncell_all * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(d.ev_atom, 0, NS * sizeof(double2), c->st));
    CK(cudaMemsetAsync(d.thermo_rep, 0, 8 * (size_t)R * sizeof(double), c->st));
    b.rep_of = drep_of;
    b.cell_rep = dcell_rep;
  }
  if (rc) return rc;
  b.rep = drep;
  b.rep_flag = dflag;
  CK(cudaMemcpyAsync(drep, c->reps.data(), R * sizeof(RepBox), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(dflag, 0, R * sizeof(int), c->st));
  // initial capacity from the densest replica: 1.4 x the mean count in the cutoff sphere, plus headroom
  double rho = 0.0;
  for (const RepBox &rb : c->reps) rho = std::max(rho, rb.natoms / (rb.L[0] * rb.L[1] * rb.L[2]));
  const double ce = c->cutoff_extra;
  const int cap = c->p.nbr_capacity > 0 ? c->p.nbr_capacity : (int)(1.4 * rho * 4.18879020479 * ce * ce * ce) + 48;
  RK(alloc_nbr(c, cap));
  if (on_device) {
    // the caller's arrays, raw, into the rebuild scratch (32 B per slot each: positions
    // and velocities 24 B, types and ids 8 B + 8 B), then converted and checked
    double *raw_pos = reinterpret_cast<double *>(d.t_pos), *raw_vel = reinterpret_cast<double *>(d.t_vel);
    uint64_t *raw_type = reinterpret_cast<uint64_t *>(d.t_acc), *raw_id = raw_type + N;
    int *type_count = d.scan_part;  // SCAN_SLICES >= CAVGPU_MAX_TYPES ints
    CK(cudaMemcpyAsync(raw_pos, pos3, 3 * sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, c->st));
    if (vel3) CK(cudaMemcpyAsync(raw_vel, vel3, 3 * sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(raw_type, type, sizeof(uint64_t) * (size_t)N, cudaMemcpyHostToDevice, c->st));
    if (id) CK(cudaMemcpyAsync(raw_id, id, sizeof(uint64_t) * (size_t)N, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(d.perm, 0, NS * sizeof(int), c->st));
    CK(cudaMemsetAsync(type_count, 0, CAVGPU_MAX_TYPES * sizeof(int), c->st));
    RK(launch_upload_single(d, b, N, c->p.ntypes, vel3 != nullptr, id != nullptr, raw_pos, raw_vel, raw_type,
                            raw_id, d.perm, type_count, c->st));
    int f[F_NWORDS];
    int counts_h[CAVGPU_MAX_TYPES];
    CK(cudaMemcpyAsync(counts_h, type_count, sizeof(counts_h), cudaMemcpyDeviceToHost, c->st));
    RK(read_flags(c, f));
    if (f[F_UPLOAD_BAD]) return CAVGPU_E_ARG;
    for (int t = 0; t < CAVGPU_MAX_TYPES; ++t) ntype[t] = counts_h[t];
  } else {
    CK(cudaMemcpyAsync(d.pos, hp.data(), NS * sizeof(dbl4), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.vel, hv.data(), NS * sizeof(dbl4), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.type, ht.data(), NS * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(d.id, hid.data(), NS * sizeof(uint32_t), cudaMemcpyHostToDevice, c->st));
  }
  CK(cudaMemsetAsync(d.acc, 0, NS * sizeof(dbl4), c->st));
  CK(cudaMemsetAsync(d.nnbr, 0, NS * sizeof(int), c->st));
  CK(cudaMemsetAsync(d.cell_count, 0, ncell_all * sizeof(int), c->st));
  CK(cudaMemsetAsync(d.cell_cursor, 0, ncell_all * sizeof(int), c->st));
  const int end_slot = NS;  // the start after the last cell (the per-replica scans never write it)
  CK(cudaMemcpyAsync(d.cell_start + ncell_all, &end_slot, sizeof(int), cudaMemcpyHostToDevice, c->st));
  double msum0 = 0.0;
  for (int t = 0; t < CAVGPU_MAX_TYPES; ++t) msum0 += c->p.mass[t] * (double)ntype[t];
  double th[8] = {0, 0, 0, 0, 0, msum0, 0, 0};
  CK(cudaMemcpyAsync(d.thermo, th, sizeof(th), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->uploaded = true;
  return CAVGPU_OK;
}

int setup_common(cavgpu_ctx *c) {
  if (!c->uploaded) return CAVGPU_E_STATE;
  RK(forced_build(c));
  RK(launch_force(c->d, c->b, c->sc, c->lc, 0, 1, 0, FUSE_NONE, 0, 0, c->st));
  c->kernel_launches += 1;
  if (c->b.nrep == 1) {
    RK(launch_thermo_final(c->d, c->tc, force_grid_blocks(c->lc), force_grid_blocks(c->lc), 0, -1, c->st));
  } else {
    RK(launch_thermo_replicas(c->d, c->b, c->tc, 1, 1, c->st));
  }
  c->kernel_launches += 1;
  RK(check_status(c));
  c->set_up = true;
  return CAVGPU_OK;
}

int ensure_status(cavgpu_ctx *c) {
  if (c->h_status) return CAVGPU_OK;
  int *h = nullptr;
  CK(cudaMallocHost(&h, 2 * F_NWORDS * sizeof(int)));
  c->h_status = h;
  for (auto &e : c->ev_status) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return CAVGPU_OK;
}

// The chunk with plan `pl` halted after completing k of its steps because step k's
// list build overflowed (the rebuild ran, its rows were cut at `cap`; the pair
// kernel did not).  Bring the gathered coordinates back to their canonical buffer,
// grow the list, build it again from the same positions -- the same cells, slot
// order and rows as an uninterrupted run with a larger list -- and complete step k:
// its pair kernel with the closing update, its thermo record, constraint::Nve.
// `g` = the step's index in the call (for the thermo record).
int complete_overflowed_step(cavgpu_ctx *c, const ChunkPlan &pl, int k, int64_t g, int64_t nsteps, int64_t every,
                             double *out5, int need) {
  if (pl.fused_before(k) & 1) {
    if (c->p.precision == CAVGPU_MIXED)
      CK(cudaMemcpyAsync(c->d.rel, c->d.rel_alt, (size_t)c->b.nslot * sizeof(float4), cudaMemcpyDeviceToDevice, c->st));
    else
      CK(cudaMemcpyAsync(c->d.pos, c->d.pos_alt, (size_t)c->b.nslot * sizeof(dbl4), cudaMemcpyDeviceToDevice, c->st));
  }
  RK(alloc_nbr(c, (int)(need * 1.25) + 32));
  RK(forced_build(c, false));
  const bool th = (every > 0 && (g + 1) % every == 0) || (every == 0 && g == nsteps - 1);
  const int ring_slot = (th && every > 0) ? 0 : -1;
  long long nl = 0;
  RK(launch_force(c->d, c->b, c->sc, c->lc, is_lang(c) ? 2 : 1, th, 0, FUSE_NONE, 0, 0, c->st));
  nl += 1;
  if (th) RK(enqueue_thermo_after_force(c, ring_slot, &nl));
  if (c->nve.step > 0 && !is_lang(c)) {
    RK(launch_nve(c->d, c->b, c->tc, c->nve, 0, th, ring_slot, c->st));
    nl += 3;
  }
  RK(launch_advance_step(c->d, c->st));
  c->kernel_launches += nl + 1;
  if (ring_slot >= 0)
    CK(cudaMemcpyAsync(out5 + THERMO_REC * ((g + 1) / every - 1), c->d.thermo_ring, THERMO_REC * sizeof(double),
                       cudaMemcpyDeviceToHost, c->st));
  return CAVGPU_OK;
}

// Steps of cavgpu_run: chunks of up to S steps (one captured graph each, cached per
// size and record period; or launched directly when steps_per_graph < 0).  Each
// chunk ends with a copy of the status words into pinned host memory; while the
// device runs chunk g the host reads the status of chunk g - 1, so a NaN or a list
// overflow is seen one chunk later at most, and the steps after it did nothing (the
// halt).  A NaN ends the call (CAVGPU_E_NAN, the state at the failing step, as the
// reference's run ends there, src/md_simulator.cpp:646-652); an overflow grows the
// list and completes the step, and the run goes on.  Without records, the call's
// last chunk computes the thermo of its final step, so that the state after the
// call carries a fresh temperature (finalize_temperature runs every step).
int run_steps(cavgpu_ctx *c, int64_t nsteps, int64_t every, double *out5) {
  int S = c->p.steps_per_graph > 0 ? std::min(c->p.steps_per_graph, MAX_GRAPH_STEPS) : 50;
  if (every > 0) S = (int)std::max<int64_t>(every, (S / every) * every);
  const bool eager = c->p.steps_per_graph < 0;
  RK(ensure_status(c));
  int f[F_NWORDS];
  RK(read_flags(c, f));
  if (f[F_NAN]) return CAVGPU_E_NAN;  // a context that met a NaN does not step again
  const int passes0 = f[F_PASSES];
  struct InFlight {
    int64_t start;
    int sz, slot;
    const ChunkPlan *plan;
  };
  std::deque<InFlight> q;
  int64_t done = 0, launched = 0;
  int slot = 0;
  const size_t depth = c->prof ? 1 : 2;  // profiling reads its events chunk by chunk
  while (done < nsteps) {
    while (launched < nsteps && q.size() < depth) {
      const int64_t left = nsteps - launched;
      int sz = (int)std::min<int64_t>(left, S), ev;
      if (every == 0) ev = (left == sz) ? sz : 0;
      else if (launched % every != 0) {  // resuming after a completed overflow step: up to the next record
        sz = (int)std::min<int64_t>(left, every - launched % every);
        ev = (launched + sz) % every == 0 ? sz : 0;
      } else if (sz % every == 0) ev = (int)every;
      else {  // a tail that holds no whole record period: one step at a time
        sz = 1;
        ev = ((launched + 1) % every == 0) ? 1 : 0;
      }
      const ChunkPlan *plan;
      if (!eager) {
        int rc = CAVGPU_OK;
        GraphEntry *g = get_graph(c, sz, ev, &rc);
        if (!g) return rc;
        CK(cudaGraphLaunch(g->exec, c->st));
        c->graph_launches += 1;
        c->kernel_launches += g->launches;
        plan = &g->plan;
      } else {
        auto it = c->eager_plans.find({sz, ev});
        if (it == c->eager_plans.end()) it = c->eager_plans.emplace(std::make_pair(sz, ev), make_plan(c, sz, ev)).first;
        plan = &it->second;
        if (c->prof) RK(ensure_events(c, sz));
        long long nl = 0;
        RK(enqueue_chunk(c, *plan, false, &nl));
        c->kernel_launches += nl;
      }
      const int nrec = ev > 0 ? sz / ev : 0;
      if (every > 0 && nrec > 0)
        CK(cudaMemcpyAsync(out5 + THERMO_REC * ((launched + ev) / every - 1), c->d.thermo_ring,
                           THERMO_REC * sizeof(double) * nrec, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(c->h_status + slot * F_NWORDS, c->d.flags, F_NWORDS * sizeof(int), cudaMemcpyDeviceToHost,
                         c->st));
      CK(cudaEventRecord(c->ev_status[slot], c->st));
      q.push_back({launched, sz, slot, plan});
      slot ^= 1;
      launched += sz;
    }
    const InFlight p = q.front();
    q.pop_front();
    CK(cudaEventSynchronize(c->ev_status[p.slot]));
    const int *hf = c->h_status + p.slot * F_NWORDS;
    c->max_nb = std::max(c->max_nb, hf[F_MAXNB]);
    if (c->prof) RK(collect_profile(c, p.sz));
    if (!hf[F_HALT]) {
      done = p.start + p.sz;
      c->steps_done += p.sz;
      continue;
    }
    // halted inside chunk p; the chunk after it, if launched, did nothing
    CK(cudaStreamSynchronize(c->st));
    q.clear();
    RK(read_flags(c, f));
    const int k = f[F_HALT_STEP];
    done = p.start + k;
    c->steps_done += k;
    if (f[F_NAN] || !f[F_OVERFLOW]) return CAVGPU_E_NAN;
    const ChunkPlan plan = *p.plan;  // growing the list frees the graphs that hold it
    RK(complete_overflowed_step(c, plan, k, done, nsteps, every, out5, f[F_OVERFLOW]));
    RK(read_flags(c, f));
    if (f[F_HALT]) return f[F_NAN] ? CAVGPU_E_NAN : CAVGPU_E_NLIST_OVERFLOW;
    done += 1;
    c->steps_done += 1;
    launched = done;
  }
  RK(check_status(c));
  // rebuild kernels launched by the graphs' conditional nodes
  if (!eager) {
    RK(read_flags(c, f));
    if (f[F_PASSES] > passes0) c->kernel_launches += (long long)rebuild_kernels(c->b) * (f[F_PASSES] - passes0);
  }
  return CAVGPU_OK;
}

}  // namespace

extern "C" {

void cavgpu_default_params(cavgpu_params *p) {
  std::memset(p, 0, sizeof(*p));
  for (int a = 0; a < 3; ++a) { p->bc[a] = 1; p->hi[a] = 1.0; }
  p->ntypes = 1;
  p->nl_cutoff = 2.5;
  p->nl_coef = 1.12347;  // Neighborlist::cutoff_extra_coef default (inc/caviar2/neighborlist.hpp:147)
  p->lj_cutoff = 2.5;
  for (int k = 0; k < CAVGPU_MAX_TYPES * CAVGPU_MAX_TYPES; ++k) { p->eps[k] = 1.0; p->sigma[k] = 1.0; }
  for (int t = 0; t < CAVGPU_MAX_TYPES; ++t) p->mass[t] = 1.0;
  p->k_b = 1.0;
  p->dt = 0.001;
  p->lang_kb = 1.0;
  p->lang_kbt = -1.0;
  p->n_r_df = 3;
  p->precision = CAVGPU_FP64;
}

const char *cavgpu_last_cuda_error(void) {
  const cudaError_t e = cudaPeekAtLastError();  // a failed kernel launch leaves its error here
  return e != cudaSuccess ? cudaGetErrorString(e) : g_last_cuda_error;
}

const char *cavgpu_strerror(int s) {
  switch (s) {
    case CAVGPU_OK: return "ok";
    case CAVGPU_E_ARG: return "invalid argument";
    case CAVGPU_E_CUDA: return "CUDA error (or no CUDA device)";
    case CAVGPU_E_NAN: return "NaN acceleration";
    case CAVGPU_E_NLIST_OVERFLOW: return "neighbour list capacity exceeded";
    case CAVGPU_E_STATE: return "call out of order";
    case CAVGPU_E_NOMEM: return "device allocation failed";
    case CAVGPU_E_RANGE: return "size beyond the stated maximum";
    default: return "unknown status";
  }
}

int cavgpu_create(const cavgpu_params *p, cavgpu_ctx **out) {
  if (!p) return CAVGPU_E_ARG;
  return create_common(p, 1, p->lo, p->hi, out);
}

int cavgpu_create_batch(const cavgpu_params *p, int32_t nrep, const double *lo3, const double *hi3,
                        cavgpu_ctx **out) {
  return create_common(p, nrep, lo3, hi3, out);
}

void cavgpu_destroy(cavgpu_ctx *c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  free_graphs(c);
  for (auto e : c->ev0) cudaEventDestroy(e);
  for (auto e : c->ev1) cudaEventDestroy(e);
  for (auto e : c->ev_status) if (e) cudaEventDestroy(e);
  if (c->h_status) cudaFreeHost(c->h_status);
  for (void *q : c->allocs) cudaFree(q);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->side) cudaStreamDestroy(c->side);
  delete c;
}

int cavgpu_upload(cavgpu_ctx *c, int64_t n, const double *pos3, const double *vel3, const uint64_t *type,
                  const uint64_t *id) {
  if (!c || n < 1 || c->b.nrep != 1) return CAVGPU_E_ARG;
  return upload_common(c, &n, pos3, vel3, type, id);
}

int cavgpu_upload_batch(cavgpu_ctx *c, const int64_t *counts, const double *pos3, const double *vel3,
                        const uint64_t *type) {
  if (!c || !counts) return CAVGPU_E_ARG;
  return upload_common(c, counts, pos3, vel3, type, nullptr);
}

int cavgpu_set_molecules(cavgpu_ctx *c, const int32_t *mol) {
  if (!c || !mol) return CAVGPU_E_ARG;
  if (!c->uploaded || c->set_up || !c->d.mol) return CAVGPU_E_STATE;
  // slots are still in upload order: replica r's atoms from its slot offset, padding -1
  std::vector<int> h(c->b.nslot, -1);
  int64_t k = 0;
  for (const RepBox &rb : c->reps)
    for (int a = 0; a < rb.natoms; ++a) h[rb.slot_off + a] = mol[k++];
  CK(cudaMemcpyAsync(c->d.mol, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return CAVGPU_OK;
}

int cavgpu_setup(cavgpu_ctx *c) {
  if (!c) return CAVGPU_E_ARG;
  return setup_common(c);
}

int cavgpu_run(cavgpu_ctx *c, int64_t nsteps, int64_t every, double *out5) {
  if (!c || nsteps < 0 || every < 0 || (every > 0 && !out5)) return CAVGPU_E_ARG;
  if (every > 0 && c->b.nrep > 1) return CAVGPU_E_ARG;  // batches: cavgpu_thermo_batch after the call
  if (!c->set_up) return CAVGPU_E_STATE;
  if (nsteps == 0) return CAVGPU_OK;
  return run_steps(c, nsteps, every, out5);
}

int cavgpu_step(cavgpu_ctx *c, int64_t nsteps) { return cavgpu_run(c, nsteps, 0, nullptr); }

int cavgpu_autotune(cavgpu_ctx *c, int32_t trial_steps, int32_t flags, int64_t *out6) {
  if (!c || trial_steps < 0) return CAVGPU_E_ARG;
  if (!c->set_up) return CAVGPU_E_STATE;
  const int T = trial_steps > 0 ? trial_steps : 40;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  const TuneKey key{dev, c->p.precision, c->p.integrator, c->b.nrep, c->natoms, c->p.ntypes, c->p.force_kernel};
  TuneChoice best{};
  bool cached = false;
  if (!(flags & CAVGPU_TUNE_FORCE)) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    for (const auto &e : g_tune_cache)
      if (e.first == key) { best = e.second; cached = true; }
  }
  // snapshot of the per-slot state and the step counters; trials run from it and
  // the chosen shape restarts from it (a forced rebuild re-derives lists and cells)
  const size_t NS = (size_t)c->b.nslot;
  dbl4 *snap = nullptr;
  int *snap_i = nullptr;
  long long snap_step = 0;
  int snap_flags[F_NWORDS];
  double snap_thermo[8];
  std::vector<double> snap_rep(c->d.thermo_rep ? 8 * (size_t)c->b.nrep : 0);
  const long long steps0 = c->steps_done, graphs0 = c->graph_launches, kern0 = c->kernel_launches;
  const bool prof0 = c->prof;
  if (cudaMalloc(&snap, 3 * NS * sizeof(dbl4)) != cudaSuccess) { cudaGetLastError(); return CAVGPU_E_NOMEM; }
  if (cudaMalloc(&snap_i, 2 * NS * sizeof(int)) != cudaSuccess) { cudaFree(snap); cudaGetLastError(); return CAVGPU_E_NOMEM; }
  // per-slot crossing counts and molecule indices move with the atoms as well
  int4 *snap_img = nullptr;
  int *snap_mol = nullptr;
  if ((c->d.img && cudaMalloc(&snap_img, NS * sizeof(int4)) != cudaSuccess) ||
      (c->d.mol && cudaMalloc(&snap_mol, NS * sizeof(int)) != cudaSuccess)) {
    cudaGetLastError();
    cudaFree(snap); cudaFree(snap_i); cudaFree(snap_img);
    return CAVGPU_E_NOMEM;
  }
  dbl4 *const src4[3] = {c->d.pos, c->d.vel, c->d.acc};
  int rc = CAVGPU_OK;
  auto save = [&]() {
    for (int k = 0; k < 3 && !rc; ++k)
      rc = cuda_rc(cudaMemcpyAsync(snap + k * NS, src4[k], NS * sizeof(dbl4), cudaMemcpyDeviceToDevice, c->st));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(snap_i, c->d.type, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(snap_i + NS, c->d.id, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    if (!rc && snap_img)
      rc = cuda_rc(cudaMemcpyAsync(snap_img, c->d.img, NS * sizeof(int4), cudaMemcpyDeviceToDevice, c->st));
    if (!rc && snap_mol)
      rc = cuda_rc(cudaMemcpyAsync(snap_mol, c->d.mol, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(&snap_step, c->d.step_base, sizeof(long long), cudaMemcpyDeviceToHost, c->st));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(snap_flags, c->d.flags, sizeof(snap_flags), cudaMemcpyDeviceToHost, c->st));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(snap_thermo, c->d.thermo, sizeof(snap_thermo), cudaMemcpyDeviceToHost, c->st));
    if (!rc && !snap_rep.empty())
      rc = cuda_rc(cudaMemcpyAsync(snap_rep.data(), c->d.thermo_rep, snap_rep.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->st));
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(c->st));
  };
  // back to the snapshot with launch shape (tpa, block, kernel): list storage for the
  // shape, state copied back, forced rebuild
  auto restore = [&](int tpa, int block, int seg) -> int {
    c->lc.tpa = tpa;
    c->lc.block = block;
    c->lc.use_seg = seg;
    c->d.tpa = tpa;
    RK(alloc_nbr(c, c->d.cap));
    for (int k = 0; k < 3; ++k)
      CK(cudaMemcpyAsync(src4[k], snap + k * NS, NS * sizeof(dbl4), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.type, snap_i, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.id, snap_i + NS, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    if (snap_img) CK(cudaMemcpyAsync(c->d.img, snap_img, NS * sizeof(int4), cudaMemcpyDeviceToDevice, c->st));
    if (snap_mol) CK(cudaMemcpyAsync(c->d.mol, snap_mol, NS * sizeof(int), cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.step_base, &snap_step, sizeof(long long), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.flags, snap_flags, sizeof(snap_flags), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->d.thermo, snap_thermo, sizeof(snap_thermo), cudaMemcpyHostToDevice, c->st));
    if (!snap_rep.empty())
      CK(cudaMemcpyAsync(c->d.thermo_rep, snap_rep.data(), snap_rep.size() * sizeof(double), cudaMemcpyHostToDevice,
                         c->st));
    RK(forced_build(c));
    int f[F_NWORDS];
    RK(read_flags(c, f));
    // the forced build is not a rebuild of the trajectory: keep the counts of the snapshot
    f[F_REBUILDS] = snap_flags[F_REBUILDS];
    f[F_PASSES] = snap_flags[F_PASSES];
    CK(cudaMemcpyAsync(c->d.flags, f, sizeof(f), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return CAVGPU_OK;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  save();
  if (!rc) rc = cuda_rc(cudaEventCreate(&e0));
  if (!rc) rc = cuda_rc(cudaEventCreate(&e1));
  c->prof = false;
  int trials = 0;
  // one trial: a warm-up graph (capture, first replay) then T steps timed on the stream
  // (an eager context, steps_per_graph < 0, stays eager: spg is then -1)
  auto trial = [&](int tpa, int block, int seg, int spg, float *ms) -> int {
    RK(restore(tpa, block, seg));
    c->p.steps_per_graph = spg;
    RK(cavgpu_run(c, spg > 0 ? std::min(T, spg) : 2, 0, nullptr));
    CK(cudaEventRecord(e0, c->st));
    RK(cavgpu_run(c, T, 0, nullptr));
    CK(cudaEventRecord(e1, c->st));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(ms, e0, e1));
    ++trials;
    return CAVGPU_OK;
  };
  const int spg0 = c->p.steps_per_graph > 0 ? c->p.steps_per_graph : (c->p.steps_per_graph < 0 ? -1 : 50);
  if (!rc && !cached) {
    float best_ms = 1e30f;
    best = {c->lc.tpa, c->lc.block, spg0, c->lc.use_seg};
    const int tpas[] = {1, 2, 4, 8};
    const int blocks[] = {64, 128, 256};
    // kernels: the mixed form tries the segment and the grid-strided kernel unless the
    // caller fixed one
    int kernels[2] = {c->lc.use_seg, -1};
    if (c->p.precision == CAVGPU_MIXED && c->p.force_kernel == CAVGPU_FORCE_AUTO) kernels[0] = 1, kernels[1] = 0;
    for (int seg : kernels) {
      if (seg < 0) break;
      for (int tpa : tpas)
        for (int block : blocks) {
          if (rc) break;
          float ms = 0.f;
          const int trc = trial(tpa, block, seg, spg0, &ms);
          if (trc == CAVGPU_E_CUDA || trc == CAVGPU_E_NOMEM) { rc = trc; break; }
          if (trc == CAVGPU_OK && ms < best_ms) { best_ms = ms; best = {tpa, block, spg0, seg}; }
        }
    }
    // graph length: the host reads status once per chunk group; longer graphs cost memory
    for (int spg : {25, 100}) {
      if (rc || spg0 < 0) break;
      float ms = 0.f;
      const int trc = trial(best.tpa, best.block, best.seg, spg, &ms);
      if (trc == CAVGPU_E_CUDA || trc == CAVGPU_E_NOMEM) { rc = trc; break; }
      if (trc == CAVGPU_OK && ms < 0.98f * best_ms) { best_ms = ms; best.spg = spg; }
    }
    if (!rc) {
      std::lock_guard<std::mutex> g(g_tune_mu);
      g_tune_cache.push_back({key, best});
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (!rc) {
    c->p.steps_per_graph = best.spg;
    rc = restore(best.tpa, best.block, best.seg);
  }
  cudaFree(snap);
  cudaFree(snap_i);
  cudaFree(snap_img);
  cudaFree(snap_mol);
  c->prof = prof0;
  c->steps_done = steps0;
  c->graph_launches = graphs0;
  c->kernel_launches = kern0;
  if (rc) return rc;
  if (out6) {
    out6[0] = best.tpa;
    out6[1] = best.block;
    out6[2] = best.spg;
    out6[3] = trials;
    out6[4] = best.seg ? CAVGPU_FORCE_SEGMENTS : CAVGPU_FORCE_STRIDED;
    out6[5] = 0;
  }
  return CAVGPU_OK;
}

int cavgpu_forces(cavgpu_ctx *c, double *virial, double *pe) {
  if (!c) return CAVGPU_E_ARG;
  if (!c->set_up) return CAVGPU_E_STATE;
  RK(forced_build(c));
  RK(launch_force(c->d, c->b, c->sc, c->lc, 0, 1, 0, FUSE_NONE, 0, 0, c->st));
  c->kernel_launches += 1;
  if (c->b.nrep == 1) {
    RK(launch_thermo_final(c->d, c->tc, force_grid_blocks(c->lc), force_grid_blocks(c->lc), 0, -1, c->st));
  } else {
    RK(launch_thermo_replicas(c->d, c->b, c->tc, 1, 1, c->st));
  }
  c->kernel_launches += 1;
  RK(check_status(c));
  if (c->b.nrep == 1) {
    double th[8];
    CK(cudaMemcpyAsync(th, c->d.thermo, sizeof(th), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (virial) *virial = th[3];
    if (pe) *pe = th[4];
  } else {  // sums over the replicas
    std::vector<double> th(8 * (size_t)c->b.nrep);
    CK(cudaMemcpyAsync(th.data(), c->d.thermo_rep, th.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    double v = 0.0, e = 0.0;
    for (int r = 0; r < c->b.nrep; ++r) { v += th[8 * r + 3]; e += th[8 * r + 4]; }
    if (virial) *virial = v;
    if (pe) *pe = e;
  }
  return CAVGPU_OK;
}

int cavgpu_thermo(cavgpu_ctx *c, double *out6) {
  if (!c || !out6) return CAVGPU_E_ARG;
  if (!c->set_up) return CAVGPU_E_STATE;
  if (c->b.nrep > 1) return CAVGPU_E_ARG;  // cavgpu_thermo_batch
  double th[8];
  int f[F_NWORDS];
  CK(cudaMemcpyAsync(th, c->d.thermo, sizeof(th), cudaMemcpyDeviceToHost, c->st));
  RK(read_flags(c, f));
  for (int k = 0; k < 5; ++k) out6[k] = th[k];
  out6[5] = (double)f[F_REBUILDS];
  return CAVGPU_OK;
}

int cavgpu_thermo_batch(cavgpu_ctx *c, double *out6) {
  if (!c || !out6) return CAVGPU_E_ARG;
  if (!c->set_up) return CAVGPU_E_STATE;
  const int R = c->b.nrep;
  if (R == 1) return cavgpu_thermo(c, out6);
  std::vector<double> th(8 * (size_t)R);
  CK(cudaMemcpyAsync(th.data(), c->d.thermo_rep, th.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int r = 0; r < R; ++r)
    for (int k = 0; k < 6; ++k) out6[6 * r + k] = th[8 * r + k];
  return CAVGPU_OK;
}

int cavgpu_download(cavgpu_ctx *c, double *pos3, double *vel3, double *acc3) {
  if (!c) return CAVGPU_E_ARG;
  if (!c->uploaded) return CAVGPU_E_STATE;
  double *outs[3] = {pos3, vel3, acc3};
  for (int w = 0; w < 3; ++w) {
    if (!outs[w]) continue;
    RK(launch_to_host_order(c->d, c->b, w, c->st));
    CK(cudaMemcpyAsync(outs[w], c->d.h3, 3 * sizeof(double) * c->natoms, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return CAVGPU_OK;
}

int cavgpu_download_images(cavgpu_ctx *c, int32_t *img3) {
  if (!c || !img3) return CAVGPU_E_ARG;
  if (!c->uploaded || !c->d.img) return CAVGPU_E_STATE;
  RK(launch_images_to_host(c->d, c->b, c->st));
  CK(cudaMemcpyAsync(img3, c->d.hi3, 3 * sizeof(int32_t) * c->natoms, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return CAVGPU_OK;
}

int64_t cavgpu_export_pairs(cavgpu_ctx *c, int32_t *out5, int64_t cap) {
  if (!c || (cap > 0 && !out5) || c->b.nrep != 1) return CAVGPU_E_ARG;
  if (!c->set_up) return CAVGPU_E_STATE;
  std::vector<int> nn(c->b.nslot);
  if (cudaMemcpyAsync(nn.data(), c->d.nnbr, c->b.nslot * sizeof(int), cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return CAVGPU_E_CUDA;
  int64_t total = 0;
  for (int v : nn) total += v;
  const int64_t take = std::min(total, cap);
  if (take <= 0) return total;
  int32_t *rows = nullptr;
  unsigned long long *cnt = nullptr;
  if (cudaMalloc(&rows, (size_t)take * 5 * sizeof(int32_t)) != cudaSuccess) { cudaGetLastError(); return CAVGPU_E_NOMEM; }
  if (cudaMalloc(&cnt, sizeof(unsigned long long)) != cudaSuccess) { cudaFree(rows); cudaGetLastError(); return CAVGPU_E_NOMEM; }
  int rc = cuda_rc(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->st));
  if (!rc) rc = launch_export_pairs(c->d, c->b, c->p.precision == CAVGPU_MIXED ? 1 : 0, rows, cnt, take, c->st);
  if (!rc) rc = cuda_rc(cudaMemcpyAsync(out5, rows, (size_t)take * 5 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
  if (!rc) rc = cuda_rc(cudaStreamSynchronize(c->st));
  cudaFree(rows);
  cudaFree(cnt);
  return rc ? rc : total;
}

int cavgpu_export_bins(cavgpu_ctx *c, int32_t *owned3, int32_t *nbins3) {
  if (!c || c->b.nrep != 1) return CAVGPU_E_ARG;
  if (!c->uploaded) return CAVGPU_E_STATE;
  if (nbins3) for (int a = 0; a < 3; ++a) nbins3[a] = c->ref_nb[a];
  if (!owned3) return CAVGPU_OK;
  RK(launch_to_host_order(c->d, c->b, 0, c->st));
  RK(launch_ref_bins(c->d, c->natoms, c->cutoff_inv, c->ref_nb, c->lo_local, c->st));
  CK(cudaMemcpyAsync(owned3, c->d.hi3, 3 * sizeof(int32_t) * c->natoms, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return CAVGPU_OK;
}

int64_t cavgpu_export_ghosts(cavgpu_ctx *c, double ghost_cutoff, int32_t *src, int32_t *shift3, double *pos3,
                             int32_t *bins3, int64_t cap) {
  if (!c || ghost_cutoff < 0.0 || c->b.nrep != 1) return CAVGPU_E_ARG;
  if (!c->uploaded) return CAVGPU_E_STATE;
  const int N = c->natoms;
  int *counts = nullptr, *starts = nullptr;
  int32_t *gs = nullptr, *gsh = nullptr, *gb = nullptr;
  double *gp = nullptr;
  const int64_t gcap = std::max<int64_t>(cap, 0);
  int rc = CAVGPU_OK;
  auto M = [&](void **q, size_t bytes) {
    if (!rc && cudaMalloc(q, std::max<size_t>(bytes, 16)) != cudaSuccess) { cudaGetLastError(); rc = CAVGPU_E_NOMEM; }
  };
  M((void **)&counts, (size_t)N * sizeof(int));
  M((void **)&starts, ((size_t)N + 1) * sizeof(int));
  M((void **)&gs, (size_t)gcap * sizeof(int32_t));
  M((void **)&gsh, (size_t)gcap * 3 * sizeof(int32_t));
  M((void **)&gp, (size_t)gcap * 3 * sizeof(double));
  M((void **)&gb, (size_t)gcap * 3 * sizeof(int32_t));
  int total = 0;
  if (!rc) rc = launch_to_host_order(c->d, c->b, 0, c->st);
  if (!rc) rc = launch_ghosts(c->d, c->b, N, ghost_cutoff, counts, starts, gs, gsh, gp, gb, gcap, c->cutoff_inv,
                              c->ref_nb, c->lo_local, c->st);
  if (!rc) rc = cuda_rc(cudaMemcpyAsync(&total, starts + N, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  if (!rc) rc = cuda_rc(cudaStreamSynchronize(c->st));
  const int64_t take = std::min<int64_t>(total, gcap);
  if (!rc && take > 0) {
    if (src) rc = cuda_rc(cudaMemcpy(src, gs, take * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (!rc && shift3) rc = cuda_rc(cudaMemcpy(shift3, gsh, take * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (!rc && pos3) rc = cuda_rc(cudaMemcpy(pos3, gp, take * 3 * sizeof(double), cudaMemcpyDeviceToHost));
    if (!rc && bins3) rc = cuda_rc(cudaMemcpy(bins3, gb, take * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  cudaFree(counts); cudaFree(starts); cudaFree(gs); cudaFree(gsh); cudaFree(gp); cudaFree(gb);
  return rc ? rc : total;
}

int cavgpu_stats(cavgpu_ctx *c, int64_t *o) {
  if (!c || !o) return CAVGPU_E_ARG;
  int f[F_NWORDS] = {0};
  if (c->uploaded) RK(read_flags(c, f));
  o[0] = c->steps_done;
  o[1] = f[F_REBUILDS];
  o[2] = std::max(c->max_nb, f[F_MAXNB]);
  o[3] = c->d.cap;
  o[4] = c->lc.tpa;
  o[5] = c->lc.block;
  o[6] = c->graph_launches;
  o[7] = c->kernel_launches;
  return CAVGPU_OK;
}

void *cavgpu_stream(cavgpu_ctx *c) { return c ? (void *)c->st : nullptr; }

int cavgpu_set_profiling(cavgpu_ctx *c, int32_t on) {
  if (!c) return CAVGPU_E_ARG;
  c->prof = on != 0;
  c->prof_ms = 0.0;
  c->prof_launches = 0;
  return CAVGPU_OK;
}

int cavgpu_read_profile(cavgpu_ctx *c, double *out2) {
  if (!c || !out2) return CAVGPU_E_ARG;
  out2[0] = (double)c->prof_launches;
  out2[1] = c->prof_ms;
  return CAVGPU_OK;
}

}  // extern "C"
