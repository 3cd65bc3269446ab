// Context and C ABI of libtpm.so (declared in include/tpm.h).
//
// The context plays the part of the reference's grid object (grid.h:14-137)
// for one box resident on one GPU: it owns every field and particle array,
// one CUDA stream, and runs the substep sequence of simulation.cpp:60-78
// (with the particle stage of simulation.cpp:64 enabled) as a fixed series of
// kernel launches with no host round trip, except that a Poisson solve with
// a positive stopping tolerance reads max|dp| back after each iteration, as
// poisson.cpp:397 decides on it.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "tpm_internal.cuh"
#include "tpm_reduce.cuh"

using tpm::Grid;
using tpm::dalloc;
using tpm::fail;
using tpm::guarded;

namespace {

const double kPreH[4] = {0.5, 0.5, 1., 1. / 6.};  // grid.cpp:18-21

bool factorable(int n) {
  if (n < 1) return false;
  for (int f : {2, 3, 5})
    while (n % f == 0) n /= f;
  return n == 1;
}

void push_scalars(tpm_ctx *c) {
  TPM_CUDA_TRY(cudaMemcpyAsync(c->dsc, c->hsc, sizeof(tpm::DevScalars), cudaMemcpyHostToDevice,
                               c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
}

void pull_scalars(tpm_ctx *c) {
  TPM_CUDA_TRY(cudaMemcpyAsync(c->hsc, c->dsc, sizeof(tpm::DevScalars), cudaMemcpyDeviceToHost,
                               c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
}

// The mixed path's post-projection residual of the last step, evaluated when
// the scalars are first read after that step (a diagnostic: the reference's
// step has none, so the step itself does not pay for it).  Its inputs - the
// projected RU (RU_int after the stage swap), the last stage's C/d^2 pairs,
// its divergence constraint and RHS mean - stay in place at the step
// boundary until the next step's Poisson right-hand side.  Not after a resume
// (no step yet) or after a call that overwrote them; queued before the read.
void div_residual_on_read(tpm_ctx *c) {
  if (c->p.precision != TPM_PREC_MIXED || c->div_every_stage || !c->stepped ||
      !c->np1_is_base || c->stage_next != 0 || c->ph_done || c->div_dirty ||
      c->div_eval_step == c->num_timestep)
    return;
  tpm::launch_div_residual(c, 3, c->RU_int);
  c->div_eval_step = c->num_timestep;
}

// device field pointer and its length in doubles
double *field_ptr(tpm_ctx *c, int f, long long *len, bool for_download) {
  const long long n = c->g.n;
  *len = n;
  bool nb = c->np1_is_base && for_download;
  switch (f) {
    case TPM_FIELD_RU: *len = 3 * n; return c->RU;
    case TPM_FIELD_RU_INT: *len = 3 * n; return c->RU_int;
    case TPM_FIELD_RU_NEW: *len = 3 * n; return c->RU_new;
    case TPM_FIELD_RU_NP1: *len = 3 * n; return nb ? c->RU : c->RU_np1;
    case TPM_FIELD_RHO: return c->Rho;
    case TPM_FIELD_RHO_INT: return c->Rho_int;
    case TPM_FIELD_RHO_NEW: return c->Rho_new;
    case TPM_FIELD_RHO_NP1: return nb ? c->Rho : c->Rho_np1;
    case TPM_FIELD_P: return c->P;
    case TPM_FIELD_C: return c->C;
    case TPM_FIELD_Q: return c->Q;
    case TPM_FIELD_FP: *len = 3 * n; return c->Fp;
    case TPM_FIELD_RHS_POIS: return c->RHS;
    case TPM_FIELD_DIVERGENCE: return c->divg;
    case TPM_FIELD_PASSIVE_SCALAR: return c->PS;  // null without solve_for_scalar
    default: return nullptr;
  }
}

// np1 copies alias the base copies after initialize / end of step; make
// them real before a caller overwrites either side.
void materialize_np1(tpm_ctx *c) {
  if (!c->np1_is_base) return;
  const long long n = c->g.n;
  TPM_CUDA_TRY(cudaMemcpyAsync(c->RU_np1, c->RU, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(c->Rho_np1, c->Rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  if (c->PS)
    TPM_CUDA_TRY(cudaMemcpyAsync(c->PS_np1, c->PS, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  for (int q = 0; q < 7 && c->np > 0; ++q)
    TPM_CUDA_TRY(cudaMemcpyAsync(c->pq[3][q], c->pq[0][q], sizeof(double) * c->np,
                                 cudaMemcpyDeviceToDevice, c->stream));
  TPM_CUDA_TRY(cudaMemcpyAsync(&c->dsc->P0_np1, &c->dsc->P0, sizeof(double), cudaMemcpyDeviceToDevice,
                               c->stream));
  c->np1_is_base = false;
}

// PARAM.update (params.cpp:80-86)
void param_update(tpm_ctx *c) {
  c->div_dirty = false;  // (a step starts: its last stage forms fresh residual inputs)
  if (c->T_cur > c->p.threshold) {
    c->Iteration = c->p.Iteration2;
    c->A = c->p.A2;
    c->gx = c->p.gx2;
    c->gy = c->p.gy2;
    c->gz = c->p.gz2;
    c->I0 = c->p.I02;
  }
}

// Captures `body` (one iteration) as the body of a conditional while node
// appended to the graph being captured on c->stream; the body's last kernel
// sets the handle (tpm::LoopCtl) to continue or stop.
template <typename F>
void capture_while(tpm_ctx *c, tpm::LoopCtl &loop, F &&body) {
  cudaStreamCaptureStatus st;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t ndeps = 0;
  TPM_CUDA_TRY(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &graph, &deps, nullptr, &ndeps));
  if (st != cudaStreamCaptureStatusActive) throw std::string("device loop outside a capture");
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = loop.handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  TPM_CUDA_TRY(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
  cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
  TPM_CUDA_TRY(cudaStreamBeginCaptureToGraph(c->side, bodyg, nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal));
  std::swap(c->stream, c->side);
  try {
    body();
  } catch (...) {
    std::swap(c->stream, c->side);
    cudaGraph_t g2 = nullptr;
    cudaStreamEndCapture(c->side, &g2);
    throw;
  }
  std::swap(c->stream, c->side);
  cudaGraph_t captured = nullptr;
  TPM_CUDA_TRY(cudaStreamEndCapture(c->side, &captured));
  TPM_CUDA_TRY(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1,
                                                   cudaStreamSetCaptureDependencies));
}

tpm::LoopCtl new_loop(tpm_ctx *c, int max_it) {
  cudaStreamCaptureStatus st;
  cudaGraph_t graph = nullptr;
  TPM_CUDA_TRY(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &graph, nullptr, nullptr, nullptr));
  tpm::LoopCtl loop;
  loop.max_it = max_it;
  TPM_CUDA_TRY(cudaGraphConditionalHandleCreate(&loop.handle, graph, 1, cudaGraphCondAssignDefault));
  return loop;
}

double read_err(tpm_ctx *c) {
  TPM_CUDA_TRY(cudaMemcpyAsync(&c->hsc->err, &c->dsc->err, sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
  TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return c->hsc->err;
}

// poisson::FFT iteration control (poisson.cpp:395-410).  Eagerly, the host
// reads max|dp| after each iteration when epsilon > 0, as the reference's loop
// does.  Inside a captured step (device_loop) the loop is a conditional while
// node whose body is one iteration; the device applies the same test, so the
// result and the iteration count are the same.  Solver = 2 runs PCG
// (tpm_pcg.cu) under the same control with its two-norm test.
void poisson_loop(tpm_ctx *c, int max_it, double eps) {
  tpm::poisson_loop_begin(c);  // skip = it = 0, err = 100
  const double eps_ctl = eps > 0 ? eps : 0.0;
  if (c->p.Solver == 2) {
    if (c->device_loop) {
      c->last_it = -1;
      tpm::LoopCtl loop = new_loop(c, max_it);
      tpm::pcg_setup(c, eps_ctl, max_it > 0 ? &loop : nullptr);
      if (max_it > 0) capture_while(c, loop, [&] { tpm::pcg_step(c, eps_ctl, &loop); });
      return;
    }
    tpm::pcg_setup(c, eps_ctl, nullptr);
    double error = eps > 0 ? read_err(c) : 100;
    int it = 0;
    while (it < max_it && error > eps) {
      tpm::pcg_step(c, eps_ctl, nullptr);
      it++;
      if (eps > 0) error = read_err(c);
    }
    c->last_it = it;
    c->total_it += it;
    if (eps > 0) c->last_err = error;
    return;
  }
  // Richardson (poisson.cpp:395-410): the device applies the reference's test
  // error > epsilon after every iteration, for any epsilon (with epsilon <= 0
  // it stops only on max|dp| == 0, turning the rest of the iterations into
  // no-ops); eagerly the host also reads max|dp| when epsilon > 0, to stop
  // launching
  const bool refine = c->p.precision == TPM_PREC_MIXED;
  if (c->device_loop) {
    c->last_it = -1;  // on the device (DevScalars::it)
    if (max_it <= 0) return;
    tpm::LoopCtl loop = new_loop(c, max_it);
    capture_while(c, loop, [&] { tpm::poisson_iteration(c, eps, &loop); });
    if (refine) tpm::refine_finish(c);
    return;
  }
  int it = 0;
  double error = 100;
  while ((it < max_it) && (error > eps)) {
    tpm::poisson_iteration(c, eps);
    it++;
    if (eps > 0) error = read_err(c);
  }
  if (refine) tpm::refine_finish(c);  // (P += dP only where the correction sum started)
  c->last_it = it;
  c->total_it += it;
  if (eps > 0) c->last_err = error;
}

// phases of one stage for the reference-granularity entry points
enum : unsigned {
  PH_P0 = 1u << 0, PH_RHO = 1u << 1, PH_PART = 1u << 2, PH_PS = 1u << 3, PH_RUWOP = 1u << 4,
  PH_DIV = 1u << 5, PH_RHSP = 1u << 6, PH_SOLVE = 1u << 7, PH_RUWP = 1u << 8, PH_MEAN = 1u << 9
};

// May phase `bit` of stage k run now?  `need`: the phases of the stage that
// the reference's loop (simulation.cpp:60-77) runs before it.
int phase_check(tpm_ctx *c, int k, unsigned bit, unsigned need, const char *name) {
  if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
  if (k < 0 || k > 3) return fail(c, TPM_ERR_ARG, std::string(name) + ": rk_stage must be 0..3");
  if (k != c->stage_next)
    return fail(c, TPM_ERR_STATE, std::string(name) + ": the context is at RK4 stage " +
                                      std::to_string(c->stage_next) + ", not " + std::to_string(k));
  if ((c->ph_done & bit) || (c->ph_done & need) != need)
    return fail(c, TPM_ERR_STATE, std::string(name) + ": out of the reference loop's order");
  return TPM_OK;
}

// the divergence constraint is kept for download (TPM_OPT_STORE_DIVERGENCE)
// and, on the mixed path, for the post-projection residual of the stages that
// evaluate it
bool store_divergence(const tpm_ctx *c, int s) {
  return c->store_div ||
         (c->p.precision == TPM_PREC_MIXED && (s == 3 || c->div_every_stage));
}

void swap_stage(tpm_ctx *c) {
  // grid::TimeAdvance_RK4 (grid.cpp:890-900): int = new
  std::swap(c->RU_int, c->RU_new);
  std::swap(c->RUi32, c->RUn32);
  std::swap(c->Rho_int, c->Rho_new);
  std::swap(c->PS_int, c->PS_new);  // grid.cpp:897
  for (int q = 0; q < 7; ++q) std::swap(c->pq[1][q], c->pq[2][q]);
  TPM_CUDA_TRY(cudaMemcpyAsync(&c->dsc->P0_int, &c->dsc->P0_new, sizeof(double),
                               cudaMemcpyDeviceToDevice, c->stream));
  c->stage_next += 1;
  c->ph_done = 0;
  c->p0_called = false;
}

// FP32 copy of RU_int for the mixed path's stencils
void refresh_rui32(tpm_ctx *c) {
  if (c->p.precision != TPM_PREC_MIXED || !c->rui32_stale) return;
  tpm::launch_to_float(c, c->RU_int, c->RUi32, 3 * c->g.n);
  c->rui32_stale = false;
}

// kernels launched while alive go to stream s (TPM_LAUNCH uses c->stream)
struct OnStream {
  tpm_ctx *c;
  cudaStream_t saved;
  OnStream(tpm_ctx *ctx, cudaStream_t s) : c(ctx), saved(ctx->stream) { c->stream = s; }
  ~OnStream() { c->stream = saved; }
};

// the auxiliary stream waits for what `stream` has enqueued so far
void aux_fork(tpm_ctx *c, cudaEvent_t e) {
  TPM_CUDA_TRY(cudaEventRecord(e, c->stream));
  TPM_CUDA_TRY(cudaStreamWaitEvent(c->aux, e, 0));
}

// `stream` waits for what the auxiliary stream has enqueued so far
void aux_join(tpm_ctx *c, cudaEvent_t e) {
  TPM_CUDA_TRY(cudaEventRecord(e, c->aux));
  TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, e, 0));
}

// One RK4 stage.  Work runs on the auxiliary stream beside the kernels it
// does not depend on (in a captured graph: parallel branches):
//   face velocity U(RU_int, Rho_int)        beside the density update (unless
//                                           the density pass forms it);
//   face coefficients C(Rho_new) (mixed)    beside the particle push and deposits
//                                           (unless the Poisson right-hand-side
//                                           pass forms them);
//   momentum deposit (its own sort scratch) beside the heat deposit (with the
//   and the momentum RHS (needs F_p)        concentration's swap).
// Each writes buffers that the kernels beside it neither read nor write; the
// stream joins back before their results are used (push, Poisson RHS).
// While per-kernel profiling is on, everything stays on one stream so that
// each kernel's events time that kernel alone.
//
// A stage runs as its head (through the particle push) and its tail; a step
// whose host transfers overlap it (tpm_step_state) captures them in separate
// graphs, and then the head joins the auxiliary stream at its end so that
// each captured piece holds whole fork/join pairs (join_aux).
template <typename F>
void beside_aux(tpm_ctx *c, int fork, F &&launch) {
  if (c->prof_on) return launch();
  aux_fork(c, c->fork_ev[fork]);
  OnStream on(c, c->aux);
  launch();
}

void stage_head(tpm_ctx *c, int s, bool join_aux) {
  refresh_rui32(c);
  const bool nb = c->np1_is_base;
  const bool par = !c->prof_on;
  auto beside = [&](int fork, auto &&launch) { beside_aux(c, fork, launch); };
  tpm::launch_p0_update(c, s);
  const bool own_u = !tpm::face_velocity_in_rho_pass(c);
  if (own_u) {
    beside(0, [&] { tpm::launch_face_velocity(c); });
    if (par) TPM_CUDA_TRY(cudaEventRecord(c->join_ev[0], c->aux));
  }
  tpm::launch_rho_update(c, s, nb);
  beside(1, [&] { tpm::launch_face_coeff(c); });
  // the FP64 push and the passive scalar read the face velocity U (the mixed
  // push interpolates RU_int / I_C2F(Rho_int) itself)
  if (par && own_u && (c->p.precision != TPM_PREC_MIXED || c->PS))
    TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join_ev[0], 0));
  tpm::launch_particle_push(c, s, nb);
  if (par && join_aux) aux_join(c, c->join_ev[1]);
}

// the tail through the Poisson solve (P final) ...
void stage_tail_solve(tpm_ctx *c, int s) {
  const bool nb = c->np1_is_base;
  const bool par = !c->prof_on;
  auto beside = [&](int fork, auto &&launch) { beside_aux(c, fork, launch); };
  beside(2, [&] {  // (F_p: the momentum deposit, then the RHS that reads it)
    tpm::particle_deposit_momentum(c);
    tpm::launch_rhs_momentum(c, s, nb);
  });
  tpm::particle_deposit_concentration(c);
  tpm::particle_heat(c);
  if (c->PS) tpm::launch_passive_scalar(c, s, nb);  // simulation.cpp:65
  if (par) aux_join(c, c->join_ev[1]);
  tpm::launch_poisson_rhs(c, s, store_divergence(c, s));
  poisson_loop(c, c->Iteration, c->p.epsilon);
}

// ... and the projection (RU_int final after it)
void stage_tail_project(tpm_ctx *c, int s) {
  tpm::launch_project(c, s);
  // (the last stage's residual is evaluated when the scalars are read)
  if (c->p.precision == TPM_PREC_MIXED && c->div_every_stage)
    tpm::launch_div_residual(c, s, c->RU_new);
  swap_stage(c);
  c->np1_is_base = false;
}

void stage_tail(tpm_ctx *c, int s) {
  stage_tail_solve(c, s);
  stage_tail_project(c, s);
}

// The tail as its particle deposits, which read neither the step's RU nor P
// (a step whose transfers overlap it runs them while those land) ...
void stage_tail_deposits(tpm_ctx *c, int s) {
  const bool par = !c->prof_on;
  auto beside = [&](int fork, auto &&launch) { beside_aux(c, fork, launch); };
  beside(2, [&] { tpm::particle_deposit_momentum(c); });
  tpm::particle_deposit_concentration(c);
  tpm::particle_heat(c);
  if (par) aux_join(c, c->join_ev[1]);
}

// ... and the rest of it (the same kernels as stage_tail, the momentum RHS on
// the step's stream)
void stage_tail_rest(tpm_ctx *c, int s) {
  const bool nb = c->np1_is_base;
  tpm::launch_rhs_momentum(c, s, nb);
  if (c->PS) tpm::launch_passive_scalar(c, s, nb);  // simulation.cpp:65
  tpm::launch_poisson_rhs(c, s, store_divergence(c, s));
  poisson_loop(c, c->Iteration, c->p.epsilon);
  stage_tail_project(c, s);
}

void substep(tpm_ctx *c, int s) {
  stage_head(c, s, false);
  stage_tail(c, s);
}

// grid::TimeAdvance (grid.cpp:595-606): the step copies base = np1; the
// particle reorder that follows may be left to the caller (reorder = false)
void time_advance(tpm_ctx *c, bool reorder = true) {
  std::swap(c->Rho, c->Rho_np1);
  std::swap(c->PS, c->PS_np1);  // grid.cpp:598
  for (int q = 0; q < 7; ++q) std::swap(c->pq[0][q], c->pq[3][q]);
  TPM_CUDA_TRY(cudaMemcpyAsync(&c->dsc->P0, &c->dsc->P0_np1, sizeof(double),
                               cudaMemcpyDeviceToDevice, c->stream));
  c->T_cur += c->p.dt;
  c->num_timestep++;
  c->np1_is_base = true;
  c->stepped = true;
  c->stage_next = 0;
  c->ph_done = 0;
  c->p0_called = false;
  if (reorder) tpm::particle_reorder(c);  // mixed path: cell order of the stage-3 positions
}

void end_step(tpm_ctx *c, bool reorder = true) {
  // simulation.cpp:80 (RU_np1.make_mean_U0) then grid::TimeAdvance
  tpm::launch_mean_reset(c);
  time_advance(c, reorder);
}

}  // namespace

namespace tpm {

void step_param_update(tpm_ctx *c) { param_update(c); }
void step_substep(tpm_ctx *c, int s) { substep(c, s); }
void step_end(tpm_ctx *c) { end_step(c); }
void step_stage_head(tpm_ctx *c, int s) { stage_head(c, s, true); }
void step_stage_tail(tpm_ctx *c, int s) { stage_tail(c, s); }
void step_stage_tail_solve(tpm_ctx *c, int s) { stage_tail_solve(c, s); }
void step_stage_tail_deposits(tpm_ctx *c, int s) { stage_tail_deposits(c, s); }
void step_stage_tail_rest(tpm_ctx *c, int s) { stage_tail_rest(c, s); }
void step_stage_tail_project(tpm_ctx *c, int s) { stage_tail_project(c, s); }
void step_end_no_reorder(tpm_ctx *c) { end_step(c, false); }

void step_body(tpm_ctx *c) {
  for (int s = 0; s < 4; ++s) substep(c, s);
  end_step(c);
}

void prof_begin(tpm_ctx *c, const char *, cudaEvent_t *ev0) {
  cudaEventCreate(ev0);
  cudaEventRecord(*ev0, c->stream);
}

void prof_end(tpm_ctx *c, const char *name, cudaEvent_t ev0) {
  cudaEvent_t ev1;
  cudaEventCreate(&ev1);
  cudaEventRecord(ev1, c->stream);
  for (auto &e : c->prof) {
    if (e.name == name) {
      e.pending.emplace_back(ev0, ev1);
      return;
    }
  }
  ProfEntry e;
  e.name = name;
  e.pending.emplace_back(ev0, ev1);
  c->prof.push_back(std::move(e));
}

}  // namespace tpm

extern "C" {

int tpm_abi_version(void) { return TPM_ABI_VERSION; }

const char *tpm_last_error(const tpm_ctx *c) { return c ? c->err.c_str() : "null context"; }

int tpm_create(const tpm_params *p, int64_t np, tpm_ctx **out) {
  if (!p || !out) return TPM_ERR_ARG;
  *out = nullptr;
  tpm_ctx *c = new (std::nothrow) tpm_ctx();
  if (!c) return TPM_ERR_NOMEM;
  c->p = *p;
  *out = c;
  if (p->elongated_box || p->solve_for_vector)
    return fail(c, TPM_ERR_UNSUPPORTED,
                "elongated box and passive vector are outside the ported path");
  if (p->precision != TPM_PREC_FP64 && p->precision != TPM_PREC_MIXED)
    return fail(c, TPM_ERR_ARG, "unknown precision");
  if (p->Solver != 0 && p->Solver != 2)
    return fail(c, TPM_ERR_UNSUPPORTED,
                "Solver must be 0 (FFT-preconditioned Richardson) or 2 (PCG)");
  if (!factorable(p->Nx) || !factorable(p->Ny) || !factorable(p->Nz) || (p->Nx % 2) ||
      p->Nx < 4 || p->Ny < 2 || p->Nz < 2)
    return fail(c, TPM_ERR_ARG, "grid sizes must be products of 2, 3, 5 with Nx even and >= 4");
  if (p->Nx / 2 > 2048 || p->Ny > 2048 || p->Nz > 2048)
    return fail(c, TPM_ERR_ARG, "FFT pencils are limited to 2048 points (Nx <= 4096, Ny, Nz <= 2048)");
  long long n = (long long)p->Nx * p->Ny * p->Nz;
  if (n >= (1LL << 31) - 1 || np < 0 || np >= (1LL << 31) - 1)
    return fail(c, TPM_ERR_ARG, "grid or particle count exceeds 2^31");
  if (!(p->dt > 0) || !(p->Lx > 0) || !(p->Ly > 0) || !(p->Lz > 0) || !(p->Mu0 > 0))
    return fail(c, TPM_ERR_ARG, "dt, box lengths and Mu0 must be positive");
  if (p->Iteration1 < 0 || p->Iteration2 < 0)
    return fail(c, TPM_ERR_ARG, "iteration counts must be >= 0");
  return guarded(c, [&]() -> int {
    TPM_CUDA_TRY(cudaGetDevice(&c->dev));
    TPM_CUDA_TRY(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->dev));
    Grid &g = c->g;
    g.nx = p->Nx; g.ny = p->Ny; g.nz = p->Nz; g.nxh = p->Nx / 2 + 1; g.sxh = g.nxh; g.n = n;
    g.mx = tpm::udiv_magic((unsigned)p->Nx); g.my = tpm::udiv_magic((unsigned)p->Ny);
    g.Lx = p->Lx; g.Ly = p->Ly; g.Lz = p->Lz;
    g.dx = p->Lx / p->Nx; g.dy = p->Ly / p->Ny; g.dz = p->Lz / p->Nz;  // gridsize.cpp:25-27
    g.inv_dx = 1. / g.dx; g.inv_dy = 1. / g.dy; g.inv_dz = 1. / g.dz;  // tensor0.cpp:17-22
    g.inv_dx2 = 1. / (g.dx * g.dx); g.inv_dy2 = 1. / (g.dy * g.dy); g.inv_dz2 = 1. / (g.dz * g.dz);
    g.idx = 1. / g.dx; g.idy = 1. / g.dy; g.idz = 1. / g.dz;          // particle.cpp:19-21
    g.xh = p->Nx * g.dx; g.yh = p->Ny * g.dy; g.zh = p->Nz * g.dz;    // gridsize.cpp:72-77
    // params.cpp:70-77
    c->R = p->Cp - p->Cv;
    c->P0ref = p->Rho0 * p->T0 * c->R;
    c->Tp = p->Rhop * p->Dp * p->Dp / (18 * p->Mu0);
    c->mp = p->Rhop * tpm::kPi * p->Dp * p->Dp * p->Dp / 6.;
    c->Vcell = g.dx * g.dy * g.dz;  // gridsize.h:43
    c->Iteration = p->Iteration1;
    c->A = p->A1; c->gx = p->gx1; c->gy = p->gy1; c->gz = p->gz1; c->I0 = p->I01;
    c->np = np;
    TPM_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    TPM_CUDA_TRY(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    TPM_CUDA_TRY(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    for (cudaEvent_t &e : c->fork_ev) TPM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t &e : c->join_ev) TPM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // fields
    c->RU = dalloc<double>(c, 3 * n); c->RU_int = dalloc<double>(c, 3 * n);
    c->RU_new = dalloc<double>(c, 3 * n); c->RU_np1 = dalloc<double>(c, 3 * n);
    c->Rho = dalloc<double>(c, n); c->Rho_int = dalloc<double>(c, n);
    c->Rho_new = dalloc<double>(c, n); c->Rho_np1 = dalloc<double>(c, n);
    c->P = dalloc<double>(c, n); c->C = dalloc<double>(c, n); c->Q = dalloc<double>(c, n);
    c->Fp = dalloc<double>(c, 3 * n); c->U = dalloc<double>(c, 3 * n);
    c->RHS = dalloc<double>(c, n); c->divg = dalloc<double>(c, n);
    c->inv_rho = dalloc<double>(c, n); c->Tgas = dalloc<double>(c, n);
    c->Cface = dalloc<double>(c, 3 * n); c->cc = dalloc<double>(c, n);
    c->spec = dalloc<double2>(c, (size_t)g.nxh * g.ny * g.nz);
    if (p->precision == TPM_PREC_MIXED) {
      c->U32 = dalloc<float>(c, 3 * n);
      c->RUi32 = dalloc<float>(c, 3 * n);
      c->RUn32 = dalloc<float>(c, 3 * n);
      c->Fp32 = dalloc<float>(c, 3 * n);
      for (float *f : {c->U32, c->RUi32, c->RUn32, c->Fp32})
        TPM_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * 3 * n, c->stream));
      c->Cs = dalloc<double>(c, 3 * n);
      TPM_CUDA_TRY(cudaMemsetAsync(c->Cs, 0, sizeof(double) * 3 * n, c->stream));
      c->Cs2 = dalloc<float2>(c, 3 * n);
      c->R0 = dalloc<float2>(c, n);
      c->cc32 = dalloc<float>(c, n);
      c->dP = dalloc<float2>(c, n);
      TPM_CUDA_TRY(cudaMemsetAsync(c->Cs2, 0, sizeof(float2) * 3 * n, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->R0, 0, sizeof(float2) * n, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->dP, 0, sizeof(float2) * n, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->cc32, 0, sizeof(float) * n, c->stream));
    }
    c->partials = dalloc<double>(c, (size_t)tpm::kPartRegions * tpm::kRedBlocks);
    c->zm_parts = dalloc<double>(c, 2 * (size_t)tpm::zm_blocks(c));
    c->dsc = dalloc<tpm::DevScalars>(c, 1);
    TPM_CUDA_TRY(cudaMemsetAsync(c->dsc, 0, sizeof(tpm::DevScalars), c->stream));
    TPM_CUDA_TRY(cudaMallocHost(&c->hsc, sizeof(tpm::DevScalars)));
    std::memset(c->hsc, 0, sizeof(tpm::DevScalars));
    for (double *f : {c->RU, c->RU_int, c->RU_new, c->RU_np1, c->Fp, c->U, c->Cface})
      TPM_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(double) * 3 * n, c->stream));
    for (double *f : {c->Rho, c->Rho_int, c->Rho_new, c->Rho_np1, c->P, c->C, c->Q, c->RHS,
                      c->divg, c->inv_rho, c->Tgas, c->cc})
      TPM_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(double) * n, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(c->partials, 0, sizeof(double) * tpm::kPartRegions * tpm::kRedBlocks,
                                 c->stream));
    c->hsc->P0 = c->hsc->P0_int = c->hsc->P0_np1 = c->hsc->P0_new = c->P0ref;
    push_scalars(c);
    tpm::fft_plans_create(c);
    tpm::rhs_kernels_setup(c);
    tpm::particle_kernels_setup(c);
    c->err_parts = dalloc<double>(c, (size_t)g.ny * g.nz);
    // particles
    for (int s = 0; s < 4; ++s)
      for (int q = 0; q < 7; ++q) {
        c->pq[s][q] = dalloc<double>(c, np);
        TPM_CUDA_TRY(cudaMemsetAsync(c->pq[s][q], 0, sizeof(double) * (np ? np : 1), c->stream));
      }
    c->rhs_t = dalloc<double>(c, np);
    TPM_CUDA_TRY(cudaMemsetAsync(c->rhs_t, 0, sizeof(double) * (np ? np : 1), c->stream));
    c->flag = dalloc<int32_t>(c, np);
    c->key_t = dalloc<int32_t>(c, np);
    c->key_r = dalloc<int32_t>(c, np);
    c->perm_t = dalloc<int32_t>(c, np);
    c->perm_r[0] = dalloc<int32_t>(c, np);
    c->starts_t = dalloc<int32_t>(c, n + 1);
    c->starts_r[0] = dalloc<int32_t>(c, n + 1);
    c->counts = dalloc<int32_t>(c, n);
    c->counts_t = dalloc<int32_t>(c, n);
    c->unsorted = dalloc<unsigned char>(c, (n + 15) / 16 * 16);
    c->unsorted_t = dalloc<unsigned char>(c, (n + 15) / 16 * 16);
    TPM_CUDA_TRY(cudaMemsetAsync(c->unsorted, 0, (n + 15) / 16 * 16, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(c->unsorted_t, 0, (n + 15) / 16 * 16, c->stream));
    c->scan_blocks = dalloc<int32_t>(c, (size_t)(n / 4096 + 2));
    c->scan_blocks_t = dalloc<int32_t>(c, (size_t)(n / 4096 + 2));
    c->pay_t = dalloc<double>(c, 6 * (size_t)np);
    c->pay_t_s = dalloc<double>(c, 6 * (size_t)np);
    c->pay_r = dalloc<double>(c, 4 * (size_t)np);
    if (p->precision == TPM_PREC_MIXED && np > 0) {  // particles kept in cell order
      c->reorder = true;
      c->pid = dalloc<int32_t>(c, np);
      c->pid2 = dalloc<int32_t>(c, np);
      c->slot = dalloc<int32_t>(c, np);
      c->flag2 = dalloc<int32_t>(c, np);
      c->rhs_t2 = dalloc<double>(c, np);
      c->pstage = dalloc<double>(c, tpm::kStateArrays * (size_t)np);
      tpm::particles_reorder_init(c);
    }
    if (p->precision == TPM_PREC_MIXED) {
      c->corner_sums = dalloc<float>(c, 16 * (size_t)n);
      c->mom_sums = dalloc<float>(c, 6 * (size_t)n);
    } else
      c->w8 = dalloc<double>(c, 16 * (size_t)np);
    c->C_next = dalloc<double>(c, n);
    if (p->Solver == 2) tpm::pcg_alloc(c);
    if (p->solve_for_scalar) {
      c->PS = dalloc<double>(c, n); c->PS_int = dalloc<double>(c, n);
      c->PS_new = dalloc<double>(c, n); c->PS_np1 = dalloc<double>(c, n);
      c->PS_face = dalloc<double>(c, 3 * n);
      for (double *f : {c->PS, c->PS_int, c->PS_new, c->PS_np1})
        TPM_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(double) * n, c->stream));
      TPM_CUDA_TRY(cudaMemsetAsync(c->PS_face, 0, sizeof(double) * 3 * n, c->stream));
      if (p->S1_type == 0) {
        // grid::C_Source (grid.cpp:718-741) with scalar_source.h: S1 = 1.*cos(1.*X)
        // at the cell centres, then S1 -= S1.mean() in tensor0::sum's order
        // (i, then j, then k innermost); time independent, so formed once here
        std::vector<double> h((size_t)n);
        for (int k = 0; k < g.nz; ++k)
          for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i) {
              const double X = g.dx / 2. + i * g.dx;
              h[((size_t)k * g.ny + j) * g.nx + i] = 1. * cos(1. * X);
            }
        double sum = 0;
        for (int i = 0; i < g.nx; ++i)
          for (int j = 0; j < g.ny; ++j)
            for (int k = 0; k < g.nz; ++k) sum += h[((size_t)k * g.ny + j) * g.nx + i];
        const double mean = sum / (double)n;
        for (double &v : h) v -= mean;
        c->S1 = dalloc<double>(c, n);
        TPM_CUDA_TRY(cudaMemcpy(c->S1, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
      }
    }
    TPM_CUDA_TRY(cudaMemsetAsync(c->C_next, 0, sizeof(double) * n, c->stream));
    TPM_CUDA_TRY(cudaMemsetAsync(c->starts_r[0], 0, sizeof(int32_t) * (n + 1), c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_destroy(tpm_ctx *c) {
  if (!c) return TPM_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto &e : c->prof)
    for (auto &ev : e.pending) {
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
  tpm::graphs_clear(c->graphs);
  tpm::graphs_clear(c->piece_graphs);
  for (void *p : c->allocs) cudaFree(p);
  if (c->fft_mem) cudaFree(c->fft_mem);
  if (c->hsc) cudaFreeHost(c->hsc);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->aux) cudaStreamDestroy(c->aux);
  if (c->io) cudaStreamDestroy(c->io);
  for (cudaEvent_t e : c->io_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->fork_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->join_ev)
    if (e) cudaEventDestroy(e);
  delete c;
  return TPM_OK;
}

int tpm_set_option(tpm_ctx *c, int option, int value) {
  return guarded(c, [&]() -> int {
    if (option == TPM_OPT_STORE_DIVERGENCE) {
      c->store_div = value != 0;
      return TPM_OK;
    }
    if (option == TPM_OPT_DIV_RESIDUAL_EVERY_STAGE) {
      c->div_every_stage = value != 0;
      return TPM_OK;
    }
    if (option == TPM_OPT_FFT_TMA) {
      c->tma_y = c->tma_z = value != 0 && c->tma_fft;
      tpm::graphs_clear(c->graphs);  // launch shapes changed
      tpm::graphs_clear(c->piece_graphs);
      return TPM_OK;
    }
    if (option == TPM_OPT_CUDA_GRAPH) {
      c->graph_mode = value != 0;
      return TPM_OK;
    }
    if (option == TPM_OPT_FUSED_DEPOSITS) {
      c->dep_fused = value != 0;
      tpm::graphs_clear(c->graphs);  // other kernels
      tpm::graphs_clear(c->piece_graphs);
      return TPM_OK;
    }
    return fail(c, TPM_ERR_ARG, "unknown option");
  });
}

int tpm_upload_field(tpm_ctx *c, int field, const double *host) {
  return guarded(c, [&]() -> int {
    if (!host) return fail(c, TPM_ERR_ARG, "null host buffer");
    if (field == TPM_FIELD_RU_NP1 || field == TPM_FIELD_RHO_NP1 || field == TPM_FIELD_RU ||
        field == TPM_FIELD_RHO)
      materialize_np1(c);
    long long len;
    double *d = field_ptr(c, field, &len, false);
    if (!d) return fail(c, TPM_ERR_ARG, "unknown field id");
    if (field == TPM_FIELD_RU_INT || field == TPM_FIELD_RU) c->rui32_stale = true;
    c->div_dirty = true;
    TPM_CUDA_TRY(cudaMemcpyAsync(d, host, sizeof(double) * len, cudaMemcpyHostToDevice, c->stream));
    if (field == TPM_FIELD_P)  // the next refinement solve starts cold
      TPM_CUDA_TRY(cudaMemsetAsync(&c->dsc->warm, 0, sizeof(int), c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_download_field(tpm_ctx *c, int field, double *host) {
  return guarded(c, [&]() -> int {
    if (!host) return fail(c, TPM_ERR_ARG, "null host buffer");
    long long len;
    double *d = field_ptr(c, field, &len, true);
    if (!d) return fail(c, TPM_ERR_ARG, "unknown field id");
    if (field == TPM_FIELD_FP && c->p.precision == TPM_PREC_MIXED)
      tpm::launch_to_double(c, c->Fp32, c->Fp, 3 * c->g.n);  // the mixed path keeps F_p in FP32
    TPM_CUDA_TRY(cudaMemcpyAsync(host, d, sizeof(double) * len, cudaMemcpyDeviceToHost, c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (field == TPM_FIELD_RHS_POIS) {
      // the kernels keep RHS_Pois un-normalised and subtract its mean where
      // they read it; apply make_mean_zero (grid.cpp:848) for the caller
      pull_scalars(c);
      const double m = c->hsc->mean_rhs;
      for (long long i = 0; i < len; ++i) host[i] -= m;
    }
    return TPM_OK;
  });
}

int tpm_upload_particles(tpm_ctx *c, int set, const double *x, const double *y, const double *z,
                         const double *u, const double *v, const double *w, const double *T,
                         const int32_t *flag) {
  return guarded(c, [&]() -> int {
    if (set < 0 || set > 3) return fail(c, TPM_ERR_ARG, "bad particle set");
    if (set == TPM_PSET_BASE || set == TPM_PSET_NP1) materialize_np1(c);
    const double *src[7] = {x, y, z, u, v, w, T};
    for (int q = 0; q < 7; ++q)
      if (src[q]) tpm::particles_from_host(c, c->pq[set][q], src[q], 8);
    if (flag) tpm::particles_from_host(c, c->flag, flag, 4);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_download_particles(tpm_ctx *c, int set, double *x, double *y, double *z, double *u,
                           double *v, double *w, double *T, int32_t *flag) {
  return guarded(c, [&]() -> int {
    if (set < 0 || set > 3) return fail(c, TPM_ERR_ARG, "bad particle set");
    int s = (set == TPM_PSET_NP1 && c->np1_is_base) ? TPM_PSET_BASE : set;
    double *dst[7] = {x, y, z, u, v, w, T};
    for (int q = 0; q < 7; ++q)
      if (dst[q]) tpm::particles_to_host(c, dst[q], c->pq[s][q], 8);
    if (flag) tpm::particles_to_host(c, flag, c->flag, 4);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_download_particle_rhs_t(tpm_ctx *c, double *rhs_t) {
  return guarded(c, [&]() -> int {
    if (!rhs_t) return fail(c, TPM_ERR_ARG, "null host buffer");
    tpm::particles_to_host(c, rhs_t, c->rhs_t, 8);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_upload_particle_rhs_t(tpm_ctx *c, const double *rhs_t) {
  return guarded(c, [&]() -> int {
    if (!rhs_t) return fail(c, TPM_ERR_ARG, "null host buffer");
    tpm::particles_from_host(c, c->rhs_t, rhs_t, 8);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_set_particle_tau(tpm_ctx *c, const double *tau) {
  return guarded(c, [&]() -> int {
    if (!tau) {
      c->tau = nullptr;
      return TPM_OK;
    }
    for (int64_t i = 0; i < c->np; ++i)
      if (!(tau[i] > 0)) return fail(c, TPM_ERR_ARG, "particle relaxation times must be > 0");
    if (!c->tau_buf) c->tau_buf = dalloc<double>(c, c->np);
    if (c->reorder && !c->tau2) c->tau2 = dalloc<double>(c, c->np);
    tpm::particles_from_host(c, c->tau_buf, tau, 8);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->tau = c->tau_buf;
    return TPM_OK;
  });
}

int tpm_set_scalars(tpm_ctx *c, double P0, double T_cur, int64_t num_timestep) {
  return guarded(c, [&]() -> int {
    pull_scalars(c);
    c->hsc->P0 = P0;
    push_scalars(c);
    c->T_cur = T_cur;
    c->num_timestep = num_timestep;
    return TPM_OK;
  });
}

int tpm_get_scalars(tpm_ctx *c, tpm_scalars *out) {
  return guarded(c, [&]() -> int {
    if (!out) return fail(c, TPM_ERR_ARG, "null output");
    div_residual_on_read(c);
    pull_scalars(c);
    out->P0 = c->hsc->P0;
    out->P0_int = c->hsc->P0_int;
    out->P0_new = c->hsc->P0_new;
    out->P0_np1 = c->np1_is_base ? c->hsc->P0 : c->hsc->P0_np1;
    out->T_cur = c->T_cur;
    out->num_timestep = c->num_timestep;
    out->last_poisson_iterations = c->hsc->it;
    out->total_poisson_iterations = c->hsc->it_sum;
    out->last_poisson_error = c->p.epsilon > 0 ? c->last_err : c->hsc->err;
    out->max_abs_div = c->p.precision == TPM_PREC_MIXED ? c->hsc->max_div : -1.0;
    if (!std::isfinite(c->hsc->mean_ru[0]) || !std::isfinite(c->hsc->mean_ru[1]) ||
        !std::isfinite(c->hsc->mean_ru[2]) || !std::isfinite(c->hsc->P0))
      return fail(c, TPM_ERR_NONFINITE, "non-finite momentum or pressure in the state");
    if (c->hsc->timeout)
      return fail(c, TPM_ERR_TIMEOUT,
                  "a kernel's bounded wait for its tile copies gave up; its results are void");
    if (c->hsc->crowded)
      return fail(c, TPM_ERR_NONFINITE,
                  "more than 65536 particles crowded into one cell (a diverging run); their "
                  "deposits were summed in arrival order");
    return TPM_OK;
  });
}

int tpm_load_state(tpm_ctx *c, const double *RU, const double *RU_int, const double *Rho,
                   const double *P, const double *const *part, const double *rhs_t, double P0,
                   double T_cur, int64_t num_timestep) {
  return guarded(c, [&]() -> int {
    if (!RU || !RU_int || !Rho || !P || (c->np > 0 && (!part || !rhs_t)))
      return fail(c, TPM_ERR_ARG, "null buffer");
    const long long n = c->g.n;
    auto up = [&](double *d, const double *h, size_t m) {
      TPM_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(double) * m, cudaMemcpyHostToDevice, c->stream));
    };
    up(c->RU, RU, 3 * n);
    up(c->RU_int, RU_int, 3 * n);
    up(c->Rho, Rho, n);
    up(c->P, P, n);
    if (c->np > 0) {
      for (int q = 0; q < 7; ++q)
        if (!part[q]) return fail(c, TPM_ERR_ARG, "null particle array");
      tpm::particle_state_from_host(c, part, rhs_t);
    }
    pull_scalars(c);  // synchronises the copies above
    c->hsc->P0 = P0;
    push_scalars(c);
    c->T_cur = T_cur;
    c->num_timestep = num_timestep;
    tpm::resume_device(c);
    return TPM_OK;
  });
}

int tpm_save_state(tpm_ctx *c, double *RU, double *RU_int, double *Rho, double *P,
                   double *const *part, double *rhs_t, tpm_scalars *sc) {
  return guarded(c, [&]() -> int {
    if (!RU || !RU_int || !Rho || !P || (c->np > 0 && (!part || !rhs_t)))
      return fail(c, TPM_ERR_ARG, "null buffer");
    if (!c->np1_is_base) return fail(c, TPM_ERR_STATE, "the state is saved at a step boundary");
    const long long n = c->g.n;
    auto down = [&](double *h, const double *d, size_t m) {
      TPM_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    };
    down(RU, c->RU, 3 * n);
    down(RU_int, c->RU_int, 3 * n);
    down(Rho, c->Rho, n);
    down(P, c->P, n);
    if (c->np > 0) {
      for (int q = 0; q < 7; ++q)
        if (!part[q]) return fail(c, TPM_ERR_ARG, "null particle array");
      tpm::particle_state_index(c);
      tpm::particle_state_stage_out(c, c->pq[0], c->rhs_t);
      tpm::particle_state_copy_out(c, part, rhs_t, c->pq[0], c->rhs_t);
    }
    div_residual_on_read(c);
    pull_scalars(c);  // synchronises the copies above
    if (sc) {
      sc->P0 = c->hsc->P0;
      sc->P0_int = c->hsc->P0_int;
      sc->P0_new = c->hsc->P0_new;
      sc->P0_np1 = c->hsc->P0;
      sc->T_cur = c->T_cur;
      sc->num_timestep = c->num_timestep;
      sc->last_poisson_iterations = c->hsc->it;
      sc->total_poisson_iterations = c->hsc->it_sum;
      sc->last_poisson_error = c->p.epsilon > 0 ? c->last_err : c->hsc->err;
      sc->max_abs_div = c->p.precision == TPM_PREC_MIXED ? c->hsc->max_div : -1.0;
    }
    return TPM_OK;
  });
}

// tpm_load_state + tpm_step + tpm_save_state in one call, the transfers
// overlapping the step.  Up (one direction of the link, in this order): the
// particle state, which the resume reads first, on the step's stream; then
// Rho and RU_int (the first stage's head) and RU and P (its tail) on a copy
// stream, the resume's particle work running meanwhile.  Down, on the copy
// stream, each result once it is final: the particle state (permuted into the
// caller's order on the step's stream) and Rho after the last stage's push,
// then P after its Poisson solve, RU_int after its projection and RU after
// the end of the step.  The step runs as seven captured pieces with the
// stream waits between them; stage 0's particle deposits, which read neither
// RU nor P, run while those two land.
int tpm_step_state(tpm_ctx *c, const double *RU, const double *RU_int, const double *Rho,
                   const double *P, const double *const *part, const double *rhs_t, double P0,
                   double T_cur, int64_t num_timestep, double *RU_out, double *RU_int_out,
                   double *Rho_out, double *P_out, double *const *part_out, double *rhs_t_out,
                   tpm_scalars *sc) {
  return guarded(c, [&]() -> int {
    if (!RU || !RU_int || !Rho || !P || !RU_out || !RU_int_out || !Rho_out || !P_out ||
        (c->np > 0 && (!part || !rhs_t || !part_out || !rhs_t_out)))
      return fail(c, TPM_ERR_ARG, "null buffer");
    for (int q = 0; q < 7 && c->np > 0; ++q)
      if (!part[q] || !part_out[q]) return fail(c, TPM_ERR_ARG, "null particle array");
    if (c->stage_next || c->ph_done)
      return fail(c, TPM_ERR_STATE, "a step is in progress through the substep or phase calls");
    if (!c->io) {
      TPM_CUDA_TRY(cudaStreamCreateWithFlags(&c->io, cudaStreamNonBlocking));
      for (cudaEvent_t &e : c->io_ev)
        TPM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const long long n = c->g.n;
    const auto up = cudaMemcpyHostToDevice, down = cudaMemcpyDeviceToHost;
    cudaEvent_t *ev = c->io_ev;
    // the copy stream's next transfers wait for event e of the step's stream
    auto io_after = [&](cudaEvent_t e) {
      TPM_CUDA_TRY(cudaEventRecord(e, c->stream));
      TPM_CUDA_TRY(cudaStreamWaitEvent(c->io, e, 0));
    };
    // 1. up: the particle state on the step's stream, then the fields on the
    // copy stream (Rho and RU_int: ev[1]; RU and P: ev[2])
    tpm::particle_state_copy_in(c, part, rhs_t);
    io_after(ev[0]);
    TPM_CUDA_TRY(cudaMemcpyAsync(c->Rho, Rho, sizeof(double) * n, up, c->io));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->RU_int, RU_int, sizeof(double) * 3 * n, up, c->io));
    TPM_CUDA_TRY(cudaEventRecord(ev[1], c->io));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->RU, RU, sizeof(double) * 3 * n, up, c->io));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->P, P, sizeof(double) * n, up, c->io));
    TPM_CUDA_TRY(cudaEventRecord(ev[2], c->io));
    tpm::particle_state_stage_in(c);
    pull_scalars(c);  // synchronises the step's stream (the copy stream goes on)
    c->hsc->P0 = P0;
    push_scalars(c);
    c->T_cur = T_cur;
    c->num_timestep = num_timestep;
    tpm::resume_device(c, ev[1]);  // reads neither RU nor P
    // 2. the step: stage 0's head, then (RU and P landed) up to stage 3's push
    tpm::step_param_update(c);
    tpm::run_piece(c, 1, false, [&] { tpm::step_stage_head(c, 0); });
    tpm::particle_state_index(c);  // (for step 3; the storage order holds until the reorder)
    tpm::run_piece(c, 2, false, [&] { tpm::step_stage_tail_deposits(c, 0); });
    TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, ev[2], 0));
    tpm::run_piece(c, 6, false, [&] {
      tpm::step_stage_tail_rest(c, 0);
      tpm::step_substep(c, 1);
      tpm::step_substep(c, 2);
      tpm::step_stage_head(c, 3);
    });
    // 3. down: the particle state (the np1 set of stage 3's push, the base
    // set after the step; in the caller's order) and Rho (Rho_np1 after
    // stage 3's density update), during stage 3's tail
    tpm::particle_state_stage_out(c, c->pq[3], c->rhs_t);
    io_after(ev[3]);
    {
      OnStream on(c, c->io);
      tpm::particle_state_copy_out(c, part_out, rhs_t_out, c->pq[3], c->rhs_t);
    }
    TPM_CUDA_TRY(cudaMemcpyAsync(Rho_out, c->Rho_np1, sizeof(double) * n, down, c->io));
    // 4. stage 3's tail in three pieces, each of P, RU_int and RU going down
    // once final
    tpm::run_piece(c, 3, false, [&] { tpm::step_stage_tail_solve(c, 3); });
    io_after(ev[4]);
    TPM_CUDA_TRY(cudaMemcpyAsync(P_out, c->P, sizeof(double) * n, down, c->io));
    tpm::run_piece(c, 4, false, [&] { tpm::step_stage_tail_project(c, 3); });
    io_after(ev[5]);
    TPM_CUDA_TRY(cudaMemcpyAsync(RU_int_out, c->RU_int, sizeof(double) * 3 * n, down, c->io));
    tpm::run_piece(c, 5, true, [&] { tpm::step_end_no_reorder(c); });
    io_after(ev[6]);
    TPM_CUDA_TRY(cudaMemcpyAsync(RU_out, c->RU, sizeof(double) * 3 * n, down, c->io));
    // 5. the reorder (the staged copies no longer read the particle sets) and
    // the step's divergence residual for the scalars
    tpm::particle_reorder(c);
    div_residual_on_read(c);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    TPM_CUDA_TRY(cudaStreamSynchronize(c->io));
    pull_scalars(c);
    if (sc) {
      sc->P0 = c->hsc->P0;
      sc->P0_int = c->hsc->P0_int;
      sc->P0_new = c->hsc->P0_new;
      sc->P0_np1 = c->hsc->P0;
      sc->T_cur = c->T_cur;
      sc->num_timestep = c->num_timestep;
      sc->last_poisson_iterations = c->hsc->it;
      sc->total_poisson_iterations = c->hsc->it_sum;
      sc->last_poisson_error = c->p.epsilon > 0 ? c->last_err : c->hsc->err;
      sc->max_abs_div = c->p.precision == TPM_PREC_MIXED ? c->hsc->max_div : -1.0;
    }
    return TPM_OK;
  });
}

int tpm_initialize(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    const long long n = c->g.n;
    // grid.cpp:461-472: stage and step copies
    TPM_CUDA_TRY(cudaMemcpyAsync(c->RU_int, c->RU, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, c->stream));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->Rho_int, c->Rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    for (int q = 0; q < 7 && c->np > 0; ++q)
      TPM_CUDA_TRY(cudaMemcpyAsync(c->pq[1][q], c->pq[0][q], sizeof(double) * c->np,
                                   cudaMemcpyDeviceToDevice, c->stream));
    pull_scalars(c);
    c->hsc->P0_int = c->hsc->P0;
    c->hsc->P0_np1 = c->hsc->P0;
    c->hsc->warm = 0;  // P comes from outside the step
    push_scalars(c);
    c->np1_is_base = true;
    c->rui32_stale = true;
    c->stage_next = 0;
    c->ph_done = 0;
    c->p0_called = false;
    if (c->PS) {  // grid.cpp:465-476
      TPM_CUDA_TRY(cudaMemcpyAsync(c->PS_int, c->PS, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
      tpm::launch_passive_scalar_face(c, c->PS);
    }
    // grid.cpp:474 (Rho_face is recomputed from Rho_int where it is needed)
    // grid.cpp:481-484: initial particle heat coupling
    c->counted_r = c->counted_t = false;  // (no push has counted the keys)
    tpm::particle_zero_fields(c);
    tpm::particle_init_heat(c);
    tpm::particle_reorder(c);
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->initialized = true;
    c->stepped = false;
    return TPM_OK;
  });
}

int tpm_resume(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    tpm::resume_device(c);
    return TPM_OK;
  });
}

}  // extern "C"

namespace tpm {

// The step-boundary state (base copies, RU_int, P, Q, rhs_t, scalars) is on
// the device; rebuild everything a step derives from it.
void resume_device(tpm_ctx *c, cudaEvent_t rho_ready) {
  {
    const long long n = c->g.n;
    // at a step boundary Rho_int == Rho, x_int == x (all particle copies
    // agree), P0_int == P0 and every np1 copy equals its base copy
    for (int q = 0; q < 7 && c->np > 0; ++q)
      TPM_CUDA_TRY(cudaMemcpyAsync(c->pq[1][q], c->pq[0][q], sizeof(double) * c->np,
                                   cudaMemcpyDeviceToDevice, c->stream));
    pull_scalars(c);
    c->hsc->P0_int = c->hsc->P0;
    c->hsc->P0_np1 = c->hsc->P0;
    c->hsc->warm = 0;  // P comes from outside the step
    push_scalars(c);
    c->np1_is_base = true;
    c->rui32_stale = true;
    c->stage_next = 0;
    c->ph_done = 0;
    c->p0_called = false;
    c->counted_r = c->counted_t = false;  // (no push has counted the keys)
    tpm::particle_resume(c);  // (the particles' heat rates and positions only)
    tpm::particle_reorder(c);
    if (rho_ready) TPM_CUDA_TRY(cudaStreamWaitEvent(c->stream, rho_ready, 0));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->Rho_int, c->Rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    if (c->PS) {
      TPM_CUDA_TRY(cudaMemcpyAsync(c->PS_int, c->PS, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
      tpm::launch_passive_scalar_face(c, c->PS);
    }
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->initialized = true;
    c->stepped = false;
  }
}

}  // namespace tpm

extern "C" {

int tpm_substep(tpm_ctx *c, int rk_stage) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (rk_stage < 0 || rk_stage > 3) return fail(c, TPM_ERR_ARG, "rk_stage must be 0..3");
    if (c->ph_done) return fail(c, TPM_ERR_STATE, "a stage is in progress through the phase calls");
    if (rk_stage == 0) c->div_dirty = false;
    substep(c, rk_stage);
    return TPM_OK;
  });
}

int tpm_end_step(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->ph_done & ~PH_MEAN)
      return fail(c, TPM_ERR_STATE, "a stage is in progress through the phase calls");
    end_step(c);
    return TPM_OK;
  });
}

// ---- the reference's grid methods one by one (simulation.cpp:58-91) ----
// Each call queues the kernels of one method of grid (grid.h:112-136) for
// RK4 stage rk_stage, on the context's stream, in the reference loop's
// order; a call out of that order returns TPM_ERR_STATE and queues nothing.
// The sequence gives the same bits as tpm_substep / tpm_end_step, which
// queue the same kernels (with independent ones on a second stream).

int tpm_param_update(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->stage_next != 0 || c->ph_done)
      return fail(c, TPM_ERR_STATE, "PARAM.update belongs at the start of a step");
    param_update(c);
    return TPM_OK;
  });
}

int tpm_update_rho(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_RHO, 0, "Update_Rho")) return rc;
    refresh_rui32(c);
    // the density pass also forms the gas temperature (P0_new/R)/Rho_new that
    // Update_Particle reads, so P0_new comes first: Update_P0 does not read
    // what Update_Rho writes (grid.cpp:816-830), so the order of the two is free
    if (!(c->ph_done & PH_P0)) {
      tpm::launch_p0_update(c, k);
      c->ph_done |= PH_P0;
    }
    tpm::launch_rho_update(c, k, c->np1_is_base);
    c->ph_done |= PH_RHO;
    return TPM_OK;
  });
}

int tpm_update_p0(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (c->initialized && k == c->stage_next && (c->ph_done & PH_P0) && !c->p0_called) {
      c->p0_called = true;  // already queued by tpm_update_rho of this stage
      return TPM_OK;
    }
    if (int rc = phase_check(c, k, PH_P0, 0, "Update_P0")) return rc;
    tpm::launch_p0_update(c, k);
    c->ph_done |= PH_P0;
    c->p0_called = true;
    return TPM_OK;
  });
}

int tpm_update_particle(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_PART, PH_P0 | PH_RHO, "Update_Particle")) return rc;
    const bool nb = c->np1_is_base;
    tpm::launch_face_velocity(c);  // U = RU_int / Rho_face (grid.cpp:868)
    tpm::launch_particle_push(c, k, nb);
    tpm::particle_deposit_momentum(c);
    tpm::particle_deposit_concentration(c);
    tpm::particle_heat(c);
    c->ph_done |= PH_PART;
    return TPM_OK;
  });
}

int tpm_update_passive_scalar(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (!c->PS) return fail(c, TPM_ERR_STATE, "solve_for_scalar is off");
    if (int rc = phase_check(c, k, PH_PS, PH_PART, "Update_Passive_Scalar")) return rc;
    tpm::launch_passive_scalar(c, k, c->np1_is_base);
    c->ph_done |= PH_PS;
    return TPM_OK;
  });
}

int tpm_update_ru_wop(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    const unsigned need = PH_PART | (c->PS ? PH_PS : 0u);
    if (int rc = phase_check(c, k, PH_RUWOP, need, "Update_RU_WOP")) return rc;
    tpm::launch_rhs_momentum(c, k, c->np1_is_base);
    c->ph_done |= PH_RUWOP;
    return TPM_OK;
  });
}

int tpm_compute_div_u_new(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_DIV, PH_RUWOP, "Compute_Div_U_new")) return rc;
    // the divergence constraint (k/Cp) Del2(1/Rho_new) - R/(Cp P0_new Vcell) Q
    // (grid.cpp:832-839) is formed by the Poisson right-hand-side pass, which
    // reads Rho_new and Q once for both; it runs at tpm_compute_rhs_pois
    c->ph_done |= PH_DIV;
    return TPM_OK;
  });
}

int tpm_compute_rhs_pois(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_RHSP, PH_DIV, "Compute_RHS_Pois")) return rc;
    tpm::launch_face_coeff(c);  // mixed path: C = 1/Rho_face pairs (grid.cpp:852)
    tpm::launch_poisson_rhs(c, k, store_divergence(c, k));
    c->ph_done |= PH_RHSP;
    return TPM_OK;
  });
}

int tpm_solve_poisson(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_SOLVE, PH_RHSP, "Solve_Poisson")) return rc;
    poisson_loop(c, c->Iteration, c->p.epsilon);
    c->ph_done |= PH_SOLVE;
    return TPM_OK;
  });
}

int tpm_update_ru_wp(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, PH_RUWP, PH_SOLVE, "Update_RU_WP")) return rc;
    tpm::launch_project(c, k);
    if (c->p.precision == TPM_PREC_MIXED && c->div_every_stage)
      tpm::launch_div_residual(c, k, c->RU_new);
    c->ph_done |= PH_RUWP;
    return TPM_OK;
  });
}

int tpm_time_advance_rk4(tpm_ctx *c, int k) {
  return guarded(c, [&]() -> int {
    if (int rc = phase_check(c, k, 0, PH_RUWP, "TimeAdvance_RK4")) return rc;
    swap_stage(c);  // next stage, no phase done
    c->np1_is_base = false;
    return TPM_OK;
  });
}

int tpm_make_mean_u0(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->stage_next != 4 || (c->ph_done & PH_MEAN))
      return fail(c, TPM_ERR_STATE, "RU_np1.make_mean_U0 belongs after the fourth stage");
    tpm::launch_mean_reset(c);
    c->ph_done |= PH_MEAN;
    return TPM_OK;
  });
}

int tpm_time_advance(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->stage_next != 4)
      return fail(c, TPM_ERR_STATE, "TimeAdvance belongs after the fourth stage");
    time_advance(c);
    return TPM_OK;
  });
}

int tpm_step(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->stage_next || c->ph_done)
      return fail(c, TPM_ERR_STATE, "a step is in progress through the substep or phase calls");
    tpm::step_any(c);
    return TPM_OK;
  });
}

int tpm_run(tpm_ctx *c, int nsteps) {
  return guarded(c, [&]() -> int {
    if (!c->initialized) return fail(c, TPM_ERR_STATE, "tpm_initialize must come first");
    if (c->stage_next || c->ph_done)
      return fail(c, TPM_ERR_STATE, "a step is in progress through the substep or phase calls");
    for (int k = 0; k < nsteps; ++k) tpm::step_any(c);
    return TPM_OK;
  });
}

int tpm_sync(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return TPM_OK;
  });
}

int tpm_poisson_solve(tpm_ctx *c, const double *C3, double *P, const double *RHS,
                      int max_iterations, double epsilon, int *iterations_out, double *error_out) {
  return guarded(c, [&]() -> int {
    if (!C3 || !P || !RHS) return fail(c, TPM_ERR_ARG, "null buffer");
    const long long n = c->g.n;
    TPM_CUDA_TRY(cudaMemcpyAsync(c->Cface, C3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->P, P, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    TPM_CUDA_TRY(cudaMemcpyAsync(c->RHS, RHS, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    pull_scalars(c);
    c->hsc->mean_rhs = 0;  // poisson::Solve uses RHS as given
    c->hsc->warm = 0;      // and starts from the caller's P
    push_scalars(c);
    tpm::launch_center_coeff_from_C(c);
    c->div_dirty = true;  // (C/d^2 and the RHS mean now belong to this solve)
    poisson_loop(c, max_iterations, epsilon);
    TPM_CUDA_TRY(cudaMemcpyAsync(P, c->P, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    pull_scalars(c);
    if (iterations_out) *iterations_out = c->hsc->it;  // the iterations the device ran
    if (error_out) *error_out = c->hsc->err;             // 100 when none ran
    return TPM_OK;
  });
}

int tpm_profile_enable(tpm_ctx *c, int on) {
  return guarded(c, [&]() -> int {
    c->prof_on = on != 0;
    return TPM_OK;
  });
}

int tpm_profile_reset(tpm_ctx *c) {
  return guarded(c, [&]() -> int {
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (auto &e : c->prof)
      for (auto &ev : e.pending) {
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
      }
    c->prof.clear();
    return TPM_OK;
  });
}

int tpm_profile_report(tpm_ctx *c, char *names, int cap, int *launches, double *total_ms,
                       int max_kernels) {
  return guarded(c, [&]() -> int {
    TPM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (auto &e : c->prof) {
      for (auto &ev : e.pending) {
        float ms = 0;
        TPM_CUDA_TRY(cudaEventElapsedTime(&ms, ev.first, ev.second));
        e.total_ms += ms;
        e.launches++;
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
      }
      e.pending.clear();
    }
    int k = 0, off = 0;
    for (auto &e : c->prof) {
      if (k >= max_kernels) break;
      int len = (int)e.name.size() + 1;
      if (names && off + len <= cap) {
        std::memcpy(names + off, e.name.c_str(), len);
        off += len;
      }
      if (launches) launches[k] = e.launches;
      if (total_ms) total_ms[k] = e.total_ms;
      ++k;
    }
    return k;
  });
}

int64_t tpm_launch_count(const tpm_ctx *c) { return c ? c->launches : 0; }

void *tpm_stream(tpm_ctx *c) { return c ? (void *)c->stream : nullptr; }

}  // extern "C"
