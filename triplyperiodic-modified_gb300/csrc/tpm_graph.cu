// Whole-step CUDA graphs, the FFT tile autotuner and batched ensembles.
//
// A step of one box is ~200 kernel launches (4 substeps, each with the
// particle stage, the momentum right-hand side and 5 kernels per Richardson
// iteration).  On a 32^3 box every kernel is a few microseconds, so an eager
// step is launch-bound; a graph replay removes the per-launch CPU cost, and a
// batch graph runs the kernel chains of many boxes concurrently, one stream
// per box, so small boxes share the 152 SMs instead of queueing.
//
// What a step launches depends only on host state (which buffer holds which
// RK copy after the pointer swaps, flags, parameters baked into kernel
// arguments): tpm::HostState.  A graph captured from one host state is
// replayed whenever the box is in that state again; the step-copy swaps
// alternate, so a run settles on two graphs per box set.  The Poisson loop's
// data-dependent stop (poisson.cpp:397) moves to the device for captured
// steps (tpm_fft.cu), so replays and eager steps give identical bits.
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "tpm_internal.cuh"

using tpm::GraphEntry;
using tpm::HostState;

namespace tpm {
namespace {

constexpr size_t kMaxGraphs = 8;  // per cache: 2 per parameter regime suffice

HostState snapshot(const tpm_ctx *c) {
  HostState h;
  std::memset(&h, 0, sizeof(h));  // padding too: states compare with memcmp
  h.RU_int = c->RU_int; h.RU_new = c->RU_new;
  h.Rho = c->Rho; h.Rho_int = c->Rho_int; h.Rho_new = c->Rho_new; h.Rho_np1 = c->Rho_np1;
  h.C = c->C; h.C_next = c->C_next;
  h.RUi32 = c->RUi32; h.RUn32 = c->RUn32;
  std::memcpy(h.pq, c->pq, sizeof(h.pq));
  h.PS = c->PS; h.PS_int = c->PS_int; h.PS_new = c->PS_new; h.PS_np1 = c->PS_np1;
  h.tau = c->tau;
  h.q_parts = c->q_parts;
  h.np1_is_base = c->np1_is_base; h.rui32_stale = c->rui32_stale; h.stepped = c->stepped;
  h.store_div = c->store_div; h.div_every_stage = c->div_every_stage;
  h.stage_next = c->stage_next; h.ph_done = (int)c->ph_done; h.p0_called = c->p0_called;
  h.counted_r = c->counted_r; h.counted_t = c->counted_t;
  h.Iteration = c->Iteration;
  std::memcpy(h.pen, c->pen, sizeof(h.pen));
  h.A = c->A; h.gx = c->gx; h.gy = c->gy; h.gz = c->gz; h.I0 = c->I0;
  return h;
}

void restore(tpm_ctx *c, const HostState &h) {
  c->RU_int = h.RU_int; c->RU_new = h.RU_new;
  c->Rho = h.Rho; c->Rho_int = h.Rho_int; c->Rho_new = h.Rho_new; c->Rho_np1 = h.Rho_np1;
  c->C = h.C; c->C_next = h.C_next;
  c->RUi32 = h.RUi32; c->RUn32 = h.RUn32;
  std::memcpy(c->pq, h.pq, sizeof(h.pq));
  c->PS = h.PS; c->PS_int = h.PS_int; c->PS_new = h.PS_new; c->PS_np1 = h.PS_np1;
  c->q_parts = h.q_parts;
  c->np1_is_base = h.np1_is_base; c->rui32_stale = h.rui32_stale; c->stepped = h.stepped;
  c->stage_next = h.stage_next; c->ph_done = (unsigned)h.ph_done; c->p0_called = h.p0_called;
  c->counted_r = h.counted_r; c->counted_t = h.counted_t;
}

bool same(const HostState &a, const HostState &b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// One step of every box: replayed from `cache` when the boxes' states match a
// captured entry, else captured (on `origin`), stored and launched.
void graph_step(const std::vector<tpm_ctx *> &boxes, cudaStream_t origin,
                std::vector<GraphEntry> &cache, cudaEvent_t fork,
                const std::vector<cudaEvent_t> &joins) {
  const size_t nb = boxes.size();
  const bool single = nb == 1 && boxes[0]->stream == origin;
  for (tpm_ctx *c : boxes) step_param_update(c);
  std::vector<HostState> pre(nb);
  for (size_t i = 0; i < nb; ++i) pre[i] = snapshot(boxes[i]);
  GraphEntry *hit = nullptr;
  for (GraphEntry &e : cache) {
    bool ok = true;
    for (size_t i = 0; i < nb && ok; ++i) ok = same(e.pre[i], pre[i]);
    if (ok) {
      hit = &e;
      break;
    }
  }
  if (hit) {
    for (size_t i = 0; i < nb; ++i) {
      tpm_ctx *c = boxes[i];
      restore(c, hit->post[i]);
      c->T_cur += c->p.dt;  // grid::TimeAdvance (grid.cpp:604-605)
      c->num_timestep++;
      c->launches += hit->launches[i];
      c->last_it = -1;
    }
  } else {
    if (cache.size() >= kMaxGraphs) {
      cudaGraphExecDestroy(cache.front().exec);
      cache.erase(cache.begin());
    }
    GraphEntry e;
    e.pre = pre;
    std::vector<double> t0(nb);
    std::vector<int64_t> n0(nb);
    for (size_t i = 0; i < nb; ++i) {
      t0[i] = boxes[i]->T_cur;
      n0[i] = boxes[i]->num_timestep;
    }
    cudaGraph_t graph = nullptr;
    TPM_CUDA_TRY(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    try {
      if (!single) TPM_CUDA_TRY(cudaEventRecord(fork, origin));
      for (size_t i = 0; i < nb; ++i) {
        tpm_ctx *c = boxes[i];
        if (!single) TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, fork, 0));
        const int64_t l0 = c->launches;
        c->device_loop = true;
        step_body(c);
        c->device_loop = false;
        e.launches.push_back(c->launches - l0);
        if (!single) {
          TPM_CUDA_TRY(cudaEventRecord(joins[i], c->stream));
          TPM_CUDA_TRY(cudaStreamWaitEvent(origin, joins[i], 0));
        }
      }
      TPM_CUDA_TRY(cudaStreamEndCapture(origin, &graph));
    } catch (...) {
      cudaGraph_t g2 = nullptr;
      cudaStreamEndCapture(origin, &g2);
      if (g2) cudaGraphDestroy(g2);
      cudaGetLastError();
      for (size_t i = 0; i < nb; ++i) {
        boxes[i]->device_loop = false;
        restore(boxes[i], pre[i]);
        boxes[i]->T_cur = t0[i];
        boxes[i]->num_timestep = n0[i];
      }
      throw;
    }
    cudaError_t err = cudaGraphInstantiate(&e.exec, graph, 0);
    cudaGraphDestroy(graph);
    TPM_CUDA_TRY(err);
    for (size_t i = 0; i < nb; ++i) e.post.push_back(snapshot(boxes[i]));
    cache.push_back(std::move(e));
    hit = &cache.back();
  }
  if (!single)  // the graph starts after work already queued on each box
    for (size_t i = 0; i < nb; ++i) {
      TPM_CUDA_TRY(cudaEventRecord(joins[i], boxes[i]->stream));
      TPM_CUDA_TRY(cudaStreamWaitEvent(origin, joins[i], 0));
    }
  TPM_CUDA_TRY(cudaGraphLaunch(hit->exec, origin));
  if (!single) {  // and later work on each box waits for it
    TPM_CUDA_TRY(cudaEventRecord(fork, origin));
    for (tpm_ctx *c : boxes) TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, fork, 0));
  }
}

double time_iterations(tpm_ctx *c, cudaEvent_t e0, cudaEvent_t e1, int reps) {
  poisson_iteration(c);  // warm-up (also loads the kernel at this tile size)
  TPM_CUDA_TRY(cudaEventRecord(e0, c->stream));
  for (int r = 0; r < reps; ++r) poisson_iteration(c);
  TPM_CUDA_TRY(cudaEventRecord(e1, c->stream));
  TPM_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  TPM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  return ms;
}

}  // namespace

void step_any(tpm_ctx *c) {
  if (c->graph_mode && !c->prof_on) {
    graph_step({c}, c->stream, c->graphs, nullptr, {});
  } else {
    step_param_update(c);
    step_body(c);
  }
}

void run_piece(tpm_ctx *c, int piece, bool advances, const std::function<void()> &body) {
  if (!c->graph_mode || c->prof_on) {
    body();
    return;
  }
  const HostState pre = snapshot(c);
  GraphEntry *hit = nullptr;
  for (GraphEntry &e : c->piece_graphs)
    if (e.piece == piece && same(e.pre[0], pre)) {
      hit = &e;
      break;
    }
  if (hit) {
    restore(c, hit->post[0]);
    if (advances) {
      c->T_cur += c->p.dt;  // grid::TimeAdvance (grid.cpp:604-605)
      c->num_timestep++;
    }
    c->launches += hit->launches[0];
    c->last_it = -1;
  } else {
    if (c->piece_graphs.size() >= 2 * kMaxGraphs) {
      cudaGraphExecDestroy(c->piece_graphs.front().exec);
      c->piece_graphs.erase(c->piece_graphs.begin());
    }
    GraphEntry e;
    e.piece = piece;
    e.pre = {pre};
    const double t0 = c->T_cur;
    const int64_t n0 = c->num_timestep, l0 = c->launches;
    cudaGraph_t graph = nullptr;
    TPM_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    try {
      c->device_loop = true;
      body();
      c->device_loop = false;
      TPM_CUDA_TRY(cudaStreamEndCapture(c->stream, &graph));
    } catch (...) {
      cudaGraph_t g2 = nullptr;
      cudaStreamEndCapture(c->stream, &g2);
      if (g2) cudaGraphDestroy(g2);
      cudaGetLastError();
      c->device_loop = false;
      restore(c, pre);
      c->T_cur = t0;
      c->num_timestep = n0;
      throw;
    }
    e.launches = {c->launches - l0};
    cudaError_t err = cudaGraphInstantiate(&e.exec, graph, 0);
    cudaGraphDestroy(graph);
    TPM_CUDA_TRY(err);
    e.post = {snapshot(c)};
    c->piece_graphs.push_back(std::move(e));
    hit = &c->piece_graphs.back();
  }
  TPM_CUDA_TRY(cudaGraphLaunch(hit->exec, c->stream));
}

void graphs_clear(std::vector<GraphEntry> &cache) {
  for (GraphEntry &e : cache)
    if (e.exec) cudaGraphExecDestroy(e.exec);
  cache.clear();
}

// Coordinate search over the pencils per block, then the threads per block,
// of the x, y and z passes.
void autotune(tpm_ctx *c) {
  const Grid &g = c->g;
  const int n_of[3] = {c->fx.n, c->fy.n, c->fz.n};
  double *P_save = dalloc<double>(c, g.n);
  DevScalars ds;
  TPM_CUDA_TRY(cudaMemcpyAsync(P_save, c->P, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(&ds, c->dsc, sizeof(ds), cudaMemcpyDeviceToHost, c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  const bool prof = c->prof_on;
  c->prof_on = false;
  TPM_CUDA_TRY(cudaMemsetAsync(&c->dsc->skip, 0, sizeof(int), c->stream));
  cudaEvent_t e0, e1;
  TPM_CUDA_TRY(cudaEventCreate(&e0));
  TPM_CUDA_TRY(cudaEventCreate(&e1));
  const int reps = 3;
  for (int d = 0; d < 3; ++d) {
    // the y and z passes of the mixed path: TMA tiles of 8 pencils (fixed
    // shape) against the best plain tiles found below; the TMA ones stay unless
    // the plain ones are clearly faster (small grids, whose Nx/2 + 1 columns
    // fill the 8-pencil tiles poorly)
    bool *tma = (d == 1) ? &c->tma_y : (d == 2) ? &c->tma_z : nullptr;
    double tma_ms = -1;
    if (tma && c->tma_fft) {
      *tma = true;
      tma_ms = time_iterations(c, e0, e1, reps);
      *tma = false;
    }
    const int cap = pens_max(n_of[d], c->p.precision == TPM_PREC_MIXED ? 8 : 16);
    int best = c->pen[d];
    double best_ms = time_iterations(c, e0, e1, reps);
    for (int cand = 1; cand <= cap; cand *= 2) {
      if (cand == best) continue;
      const int keep = c->pen[d];
      c->pen[d] = cand;
      const double ms = time_iterations(c, e0, e1, reps);
      if (ms < 0.97 * best_ms) {  // keep the incumbent unless clearly faster
        best_ms = ms;
        best = cand;
      }
      c->pen[d] = keep;
    }
    c->pen[d] = best;
    int best_t = c->fthreads[d];
    for (int th : {128, 256, 512}) {
      if (th == best_t) continue;
      const int keep = c->fthreads[d];
      c->fthreads[d] = th;
      const double ms = time_iterations(c, e0, e1, reps);
      if (ms < 0.97 * best_ms) {
        best_ms = ms;
        best_t = th;
      }
      c->fthreads[d] = keep;
    }
    c->fthreads[d] = best_t;
    if (tma_ms >= 0) *tma = !(best_ms < 0.97 * tma_ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->prof_on = prof;
  TPM_CUDA_TRY(cudaMemcpyAsync(c->P, P_save, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(c->dsc, &ds, sizeof(ds), cudaMemcpyHostToDevice, c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
}

}  // namespace tpm

// ------------------------------------------------------------------ batch
struct tpm_batch {
  std::vector<tpm_ctx *> boxes;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<GraphEntry> graphs;
  std::string err;
};

namespace {

int batch_fail(tpm_batch *b, int code, const std::string &msg) {
  if (b) b->err = msg;
  return code;
}

template <typename F>
int batch_guarded(tpm_batch *b, F &&f) {
  if (!b) return TPM_ERR_ARG;
  try {
    return f();
  } catch (const std::pair<int, std::string> &e) {
    return batch_fail(b, e.first, e.second);
  } catch (const std::string &s) {
    return batch_fail(b, TPM_ERR_CUDA, s);
  } catch (const std::bad_alloc &) {
    return batch_fail(b, TPM_ERR_NOMEM, "host allocation failed");
  }
}

// a box's error (from a tpm_* call on it) as the batch's
int box_rc(tpm_batch *b, int i, int rc) {
  if (rc != TPM_OK) b->err = "box " + std::to_string(i) + ": " + tpm_last_error(b->boxes[i]);
  return rc;
}

}  // namespace

extern "C" {

int tpm_autotune(tpm_ctx *c, int *pens_out) {
  return tpm::guarded(c, [&]() -> int {
    tpm::autotune(c);
    tpm::graphs_clear(c->graphs);  // launch shapes changed
    tpm::graphs_clear(c->piece_graphs);
    if (pens_out)
      for (int d = 0; d < 3; ++d) {
        pens_out[d] = c->pen[d];
        pens_out[3 + d] = c->fthreads[d];
      }
    return TPM_OK;
  });
}

int tpm_set_fft_tiles(tpm_ctx *c, const int *tiles) {
  return tpm::guarded(c, [&]() -> int {
    if (!tiles) return tpm::fail(c, TPM_ERR_ARG, "null tiles");
    const int n_of[3] = {c->fx.n, c->fy.n, c->fz.n};
    const int elem = c->p.precision == TPM_PREC_MIXED ? 8 : 16;
    for (int d = 0; d < 3; ++d) {
      const int p = tiles[d], t = tiles[3 + d];
      if (p < 1 || (p & (p - 1)) || p > tpm::pens_max(n_of[d], elem))
        return tpm::fail(c, TPM_ERR_ARG, "pencils per block must be a power of two within the "
                                         "pass's shared memory");
      if (t < 32 || t > 1024 || t % 32)
        return tpm::fail(c, TPM_ERR_ARG, "threads per block must be a multiple of 32, 32..1024");
    }
    for (int d = 0; d < 3; ++d) {
      c->pen[d] = tiles[d];
      c->fthreads[d] = tiles[3 + d];
    }
    tpm::graphs_clear(c->graphs);  // launch shapes changed
    tpm::graphs_clear(c->piece_graphs);
    return TPM_OK;
  });
}

int tpm_batch_create(const tpm_params *params, const int64_t *np, int nboxes, tpm_batch **out) {
  if (!params || !np || !out || nboxes < 1) return TPM_ERR_ARG;
  *out = nullptr;
  tpm_batch *b = new (std::nothrow) tpm_batch;
  if (!b) return TPM_ERR_NOMEM;
  for (int i = 0; i < nboxes; ++i) {
    tpm_ctx *c = nullptr;
    int rc = tpm_create(&params[i], np[i], &c);
    if (rc != TPM_OK) {
      if (c) tpm_destroy(c);
      tpm_batch_destroy(b);
      return rc;
    }
    b->boxes.push_back(c);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    tpm_batch_destroy(b);
    return TPM_ERR_CUDA;
  }
  b->joins.resize(nboxes, nullptr);
  for (auto &e : b->joins)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      tpm_batch_destroy(b);
      return TPM_ERR_CUDA;
    }
  *out = b;
  return TPM_OK;
}

int tpm_batch_destroy(tpm_batch *b) {
  if (!b) return TPM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  tpm::graphs_clear(b->graphs);
  for (tpm_ctx *c : b->boxes) tpm_destroy(c);
  for (cudaEvent_t e : b->joins)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return TPM_OK;
}

const char *tpm_batch_last_error(const tpm_batch *b) { return b ? b->err.c_str() : "null batch"; }

tpm_ctx *tpm_batch_box(tpm_batch *b, int i) {
  if (!b || i < 0 || i >= (int)b->boxes.size()) return nullptr;
  return b->boxes[i];
}

int tpm_batch_autotune(tpm_batch *b) {
  return batch_guarded(b, [&]() -> int {
    std::map<std::vector<int>, std::vector<int>> done;  // (nx, ny, nz, precision) -> pens
    for (size_t i = 0; i < b->boxes.size(); ++i) {
      tpm_ctx *c = b->boxes[i];
      std::vector<int> key = {c->g.nx, c->g.ny, c->g.nz, c->p.precision};
      auto it = done.find(key);
      if (it != done.end()) {
        for (int d = 0; d < 3; ++d) {
          c->pen[d] = it->second[d];
          c->fthreads[d] = it->second[3 + d];
        }
        continue;
      }
      int pens[6];
      if (int rc = box_rc(b, (int)i, tpm_autotune(c, pens))) return rc;
      done[key] = {pens[0], pens[1], pens[2], pens[3], pens[4], pens[5]};
    }
    tpm::graphs_clear(b->graphs);
    return TPM_OK;
  });
}

int tpm_batch_run(tpm_batch *b, int nsteps, int use_graph) {
  return batch_guarded(b, [&]() -> int {
    for (size_t i = 0; i < b->boxes.size(); ++i)
      if (!b->boxes[i]->initialized)
        return batch_fail(b, TPM_ERR_STATE, "box " + std::to_string(i) + " is not initialised");
    for (int k = 0; k < nsteps; ++k) {
      if (use_graph) {
        for (size_t i = 0; i < b->boxes.size(); ++i)
          if (b->boxes[i]->prof_on)
            return batch_fail(b, TPM_ERR_STATE, "profiling is on in box " + std::to_string(i));
        tpm::graph_step(b->boxes, b->stream, b->graphs, b->fork, b->joins);
      } else {
        for (size_t i = 0; i < b->boxes.size(); ++i)
          if (int rc = box_rc(b, (int)i, tpm_step(b->boxes[i]))) return rc;
      }
    }
    return TPM_OK;
  });
}

int tpm_batch_sync(tpm_batch *b) {
  return batch_guarded(b, [&]() -> int {
    TPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (tpm_ctx *c : b->boxes) TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

}  // extern "C"
