// Internal declarations shared by the CUDA translation units of libtpm.so.
//
// Data layout in HBM (one context = one periodic box):
//  * scalar fields: unghosted FP64 [Nz][Ny][Nx], x fastest, index
//    c = (k*Ny + j)*Nx + i; a neighbour index wraps periodically (this is
//    what the reference's ghost layers + halo exchange do on one rank);
//  * vector (face) fields: the x, y, z components as three such blocks back
//    to back, exactly the reference's tensor1 file layout;
//  * spectrum: half-complex [Nz][Ny][Nx/2+1] (R2C along x);
//  * particles: SoA, one array per quantity and per RK copy
//    (base, int, new, np1 as in particle.h:61-113).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "tpm.h"
#include "tpm_index.cuh"

namespace tpm {

constexpr double kPi = 3.141592653589793;  // params.h:5

struct Grid {
  int nx, ny, nz, nxh;  // nxh = nx/2 + 1 (half spectrum)
  int sxh;              // row pitch of the half spectrum in elements (>= nxh)
  long long n;          // cells
  unsigned long long mx, my;  // udiv_magic(nx), udiv_magic(ny)
  double dx, dy, dz;
  double inv_dx, inv_dy, inv_dz, inv_dx2, inv_dy2, inv_dz2;  // tensor0.cpp:17-22
  double idx, idy, idz;                                      // particle.cpp:19-21
  double Lx, Ly, Lz, xh, yh, zh;                             // gridsize.cpp:72-77
};

__host__ __device__ __forceinline__ int wrap_p(int i, int n) { return i + 1 == n ? 0 : i + 1; }
__host__ __device__ __forceinline__ int wrap_m(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__host__ __device__ __forceinline__ int wrap_any(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

#if defined(__CUDACC__)
// (i, j, k) of the flat cell index c = (k*Ny + j)*Nx + i, by the division
// magics of the grid (c < 2^31)
__device__ __forceinline__ void cell_ijk(const Grid &g, long long c, int &i, int &j, int &k) {
  const unsigned cu = (unsigned)c, t = udiv(cu, g.mx), kk = udiv(t, g.my);
  i = (int)(cu - t * (unsigned)g.nx);
  j = (int)(t - kk * (unsigned)g.ny);
  k = (int)kk;
}

// (j, k) of a pencil row r = k*Ny + j
__device__ __forceinline__ void row_jk(const Grid &g, long long r, int &j, int &k) {
  const unsigned ru = (unsigned)r, kk = udiv(ru, g.my);
  j = (int)(ru - kk * (unsigned)g.ny);
  k = (int)kk;
}
#endif

// Scalars that live on the device so a whole substep runs without host
// round trips (grid.h:100-105).
struct DevScalars {
  double P0, P0_int, P0_new, P0_np1;
  double T_scale;    // P0_new / R   (grid.cpp:882)
  double coef_div;   // -R/(Cp*P0_new*Vcell)  (grid.cpp:838)
  double mean_Q;     // mean(RHS_Part_Temp) of the current substep
  double mean_rhs;   // mean(RHS_Pois) (grid.cpp:848)
  double err;        // max|dp| of the last Poisson iteration (poisson.cpp:407)
  double mean_ru[3]; // RU_np1 component means (simulation.cpp:80)
  double max_div;    // FP64 post-projection residual (mixed path)
  double tke2;       // mean(U^2) of the last stage before projection (grid.cpp:911)
  int nonfinite;
  // set (and kept) when a kernel's bounded wait on its tile copies gave up
  int timeout;
  // Poisson iteration control on the device (graph-captured steps): `skip`
  // turns the remaining captured iterations of a solve into no-ops once
  // max|dp| <= epsilon (poisson.cpp:397); `it` counts the iterations run by
  // the current solve, `it_sum` all iterations since create.
  int skip;
  int it;
  int it_sum;
  // set (and kept) when a cell held more particles than the counting sort
  // orders (kSortMaxRun): only a diverging run crowds its particles so
  int crowded;
  // bits of max|dp| of the running Poisson iteration (the blocks' atomic
  // maximum; zero between iterations)
  unsigned long long err_acc;
  // mixed path: 1 once a refinement solve has run since P was last set from
  // outside the step (initialise, resume, upload, operator-level solve);
  // a warm solve forms one direct residual of P, a cold one two
  int warm;
};

// 1-D FFT plan in device memory: radices and exp(-2 pi i m / n) twiddles,
// and multiply-high magic numbers (ceil(2^32/d), 0 for d = 1) for the integer
// divisions of the pencil passes: by the span p of each stage, by n, 2n and
// n + 1 (the real-to-complex x pass holds rows of 2n reals and n + 1 modes).
struct FftPlan {
  int n;
  int nst;
  int radix[16];
  unsigned pmag[16];
  unsigned nmag, n2mag, nhmag;
  const double2 *tw64;  // n entries
  const float2 *tw32;   // n entries
};

// Deterministic reductions: each reducing kernel writes one partial per
// block; a one-block kernel finishes them in a fixed order.
constexpr int kRedBlocks = 1024;

struct ProfEntry {
  std::string name;
  int launches = 0;
  double total_ms = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};

// Host-side state that decides what a step launches: the buffers each role
// points at (the RK and step copies are pointer swaps), the flags and the
// parameters baked into kernel arguments.  A CUDA graph captured from one
// state replays correctly exactly when the context is in that state again.
struct HostState {
  double *RU_int, *RU_new, *Rho, *Rho_int, *Rho_new, *Rho_np1, *C, *C_next;
  float *RUi32, *RUn32;
  double *pq[4][7];
  double *PS, *PS_int, *PS_new, *PS_np1;
  const double *tau;
  int q_parts;
  int np1_is_base, rui32_stale, stepped, store_div, div_every_stage;
  int stage_next, ph_done, p0_called, counted_r, counted_t;  // (mid-step pieces)
  int Iteration;
  int pen[3];
  double A, gx, gy, gz, I0;
};

// TMA tensor maps of one FP64 device array seen as [layers][ny][nx], with
// boxes of a 32 x 8 tile, a 32 x 1 row and a 2 x 8 column pair (tpm_tma.cuh)
struct TmaField {
  const double *base = nullptr;
  long long layers = 0;
  CUtensorMap tile, row, col;
};

// One captured step of one or more boxes, with the host states before and
// after it (one per box) and the kernels it launches per box.
struct GraphEntry {
  std::vector<HostState> pre, post;
  std::vector<int64_t> launches;
  cudaGraphExec_t exec = nullptr;
  int piece = 0;  // the piece of a split step (tpm_step_state), 0 for a whole step
};

}  // namespace tpm

// The context (opaque to callers, see tpm.h).
struct tpm_ctx {
  tpm_params p;
  tpm::Grid g;
  int64_t np = 0;
  int dev = 0;
  int sms = 0;  // SM count of the device
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // captures the body of a conditional (while) graph node
  // a second stream for the kernels of a stage that do not depend on the
  // ones beside them (face velocity, face coefficients, momentum RHS), with
  // the events that fork it from and join it to `stream`
  cudaStream_t aux = nullptr;
  cudaEvent_t fork_ev[3] = {nullptr, nullptr, nullptr}, join_ev[2] = {nullptr, nullptr};
  std::string err;
  int64_t launches = 0;

  // derived constants (params.cpp:70-77)
  double R = 0, Tp = 0, mp = 0, Vcell = 0, P0ref = 0;
  // parameters switched at T_cur > threshold (params.cpp:80-86)
  double A = 0, gx = 0, gy = 0, gz = 0, I0 = 0;
  int Iteration = 0;

  double T_cur = 0;
  int64_t num_timestep = 0;
  bool initialized = false;
  bool np1_is_base = true;  // np1 copies equal base (after initialize / end of step)
  bool stepped = false;     // a full step has run since initialize / resume
  // the reference-granularity phase entry points (tpm_update_rho ...): the
  // RK4 stage the next phase belongs to (0..3; 4 once the fourth stage has
  // advanced, until the end of the step) and the phases done in it
  int stage_next = 0;
  unsigned ph_done = 0;
  bool p0_called = false;  // tpm_update_p0 was called in this stage
  int last_it = 0, total_it = 0;
  double last_err = 0;

  // ---- fields (device) ----
  double *RU = nullptr, *RU_int = nullptr, *RU_new = nullptr, *RU_np1 = nullptr;  // 3n each
  double *Rho = nullptr, *Rho_int = nullptr, *Rho_new = nullptr, *Rho_np1 = nullptr;
  double *P = nullptr, *C = nullptr, *Q = nullptr, *Fp = nullptr /*3n*/, *U = nullptr /*3n*/;
  // inv_rho = 1/Rho_new: doubles on the FP64 path, float-float pairs (one
  // float2 per cell in the same bytes) on the mixed path
  double *RHS = nullptr, *divg = nullptr, *inv_rho = nullptr, *Tgas = nullptr;
  double *Cface = nullptr /*3n*/, *cc = nullptr;
  // FP32 copies read by the FP32 stencils of the mixed path (written once per
  // value: FP64<->FP32 conversions issue on the FP64 pipe)
  float *U32 = nullptr, *RUi32 = nullptr, *RUn32 = nullptr, *Fp32 = nullptr;  // 3n each
  double *Cs = nullptr;     // 3n: C/d^2 for the mixed PCG operator
  // mixed Richardson refinement: C/d^2 per face and the base residual of the
  // correction form as float-float pairs (hi, lo), cc in FP32, and the
  // solve's correction sum (P += dP once the loop ends)
  float2 *Cs2 = nullptr;    // 3n
  float2 *R0 = nullptr;     // n
  float *cc32 = nullptr;    // n
  float2 *dP = nullptr;     // n
  bool rui32_stale = true;
  double2 *spec = nullptr;
  double *partials = nullptr;  // kRedBlocks * 4
  double *zm_parts = nullptr;  // 2 * zm_blocks: the mixed Poisson RHS's mean and TKE partials
  tpm::DevScalars *dsc = nullptr;
  tpm::DevScalars *hsc = nullptr;  // pinned mirror
  double *ax = nullptr, *ay = nullptr, *az = nullptr;  // modified wave number tables
  // 1/(ax[kx] + ay[ky] + az[kz]) per half-spectrum mode (1 at the zero mode),
  // double on the FP64 path and float on the mixed path
  void *inv_mwn = nullptr;
  tpm::FftPlan fx, fy, fz;        // FP64 passes (radices 4, 2, 3, 5)
  tpm::FftPlan fx32, fy32, fz32;  // FP32 passes (radices 16 and 8 first)
  const double2 *r2c64 = nullptr;
  const float2 *r2c32 = nullptr;
  double *err_parts = nullptr;  // one max|dp| per x-pass block (sized for one row per block)
  int pen[3] = {1, 1, 1};       // FFT pencils per block of the x, y, z passes (autotuned)
  int fthreads[3] = {256, 256, 256};  // threads per block of the x, y, z passes (autotuned)
  bool device_loop = false;     // Poisson stopping test on the device (no host read)
  void *fft_mem = nullptr;

  // ---- particles (device) ----
  double *pq[4][7] = {};  // [set][quantity] set: base,int,new,np1; q: x,y,z,u,v,w,T
  double *rhs_t = nullptr, *tau = nullptr, *tau_buf = nullptr;
  int32_t *flag = nullptr;
  int32_t *key_t = nullptr, *key_r = nullptr;
  int32_t *perm_t = nullptr, *perm_r[1] = {nullptr};
  int32_t *starts_t = nullptr, *starts_r[1] = {nullptr};
  // the counting sorts' scratch, one set per sort (the momentum deposit's
  // sort, _t, runs beside the heat deposit's): per-cell counts, the cells the
  // scatter left out of order (n rounded up to 16; all zero between sorts),
  // the scan's chunk totals
  int32_t *counts = nullptr, *counts_t = nullptr;
  unsigned char *unsorted = nullptr, *unsorted_t = nullptr;
  int32_t *scan_blocks = nullptr, *scan_blocks_t = nullptr;
  // the push has counted key_r / key_t into counts / counts_t (the next sort
  // of each skips its histogram pass)
  bool counted_r = false, counted_t = false;
  double *pay_t = nullptr, *pay_t_s = nullptr;          // 6*np
  double *pay_r = nullptr;  // 4*np: round-indexed fractions and heat rate, unsorted
  // mixed path: particles kept in cell order (particle_reorder).  pid[s] is the
  // caller's index of the particle in storage slot s; host transfers of
  // per-particle data go through it.  pid2 / flag2 / rhs_t2 / tau2 take the
  // permuted copies, pstage (kStateArrays slots of np doubles) stages the
  // caller-ordered arrays (one array in its first slot, the particle state in
  // all of them).
  bool reorder = false;
  int32_t *pid = nullptr, *pid2 = nullptr, *flag2 = nullptr;
  int32_t *slot = nullptr;  // slot[i]: storage slot of caller particle i (particle_state_index)
  double *rhs_t2 = nullptr, *tau2 = nullptr, *pstage = nullptr;
  double *w8 = nullptr;  // 16*np corner weights (heat, concentration; sorted order)
  float *corner_sums = nullptr;  // mixed: 16*n per-source-cell corner sums (heat, conc.)
  float *mom_sums = nullptr;     // mixed: 6*n per-source-cell momentum sums
  double *C_next = nullptr;  // concentration at this x_new = next substep's x_int
  // passive scalar (solve_for_scalar): RK copies, face values I_C2F(PS_new)
  // of the last stage, and the mean-free source field of S1_type 0
  double *PS = nullptr, *PS_int = nullptr, *PS_new = nullptr, *PS_np1 = nullptr;
  double *PS_face = nullptr /*3n*/, *S1 = nullptr;
  int q_parts = 1;  // number of valid partial sums of Q (heat deposit blocks)

  bool store_div = false;
  bool div_every_stage = false;
  // The mixed path's post-projection residual of a step is evaluated when the
  // scalars are first read after it (div_residual_on_read), from inputs that
  // stay in place until the next step's Poisson right-hand side: the step
  // count it was last evaluated at, and whether a call since the step has
  // overwritten its inputs (a field upload, an operator-level solve).
  int64_t div_eval_step = -1;
  bool div_dirty = false;
  bool dep_fused = true;  // TPM_OPT_FUSED_DEPOSITS
  // mixed path: the face coefficients and the Poisson right-hand side in one
  // TMA-fed z-marching pass (grids of whole 32 x 8 tiles, Solver 0), with the
  // tensor maps of the arrays it reads
  bool tma_rhs = false;
  std::vector<tpm::TmaField> tma_fields;
  // mixed path: the spectrum of the Richardson loop has rows padded to an
  // even number of float2 (a 16-byte multiple) so that the y and z pencil
  // passes move their tiles by TMA (tensor maps of the y and z tiles)
  int spec_pitch = 0;
  bool tma_fft = false;  // the y and z passes can take TMA tiles (mixed path, pencils <= 256)
  bool tma_y = false, tma_z = false;  // ... and do (on by default; the autotuner may turn one off)
  int tma_fft_blocks[2] = {0, 0};  // persistent blocks of the y and z passes
  CUtensorMap fft_map_y, fft_map_z;

  // ---- PCG pressure solve (Solver = 2; allocated on first use) ----
  double *pcg_r = nullptr, *pcg_z = nullptr, *pcg_p = nullptr, *pcg_q = nullptr;
  double *pcg_s = nullptr;  // 1/sqrt(C at the cell centre) = sqrt(-cc)
  double *pcg_sc = nullptr, *pcg_parts = nullptr;

  // ---- CUDA graph replay of whole steps (tpm_graph.cu) ----
  bool graph_mode = false;
  std::vector<tpm::GraphEntry> graphs;
  std::vector<tpm::GraphEntry> piece_graphs;  // the pieces of split steps
  // tpm_step_state: its copy stream and the events between it and the step
  cudaStream_t io = nullptr;
  cudaEvent_t io_ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};

  // ---- diagnostics (allocated on first use; tpm_diag.cu) ----
  double *diag_u = nullptr;      // 3n: face velocity RU/I_C2F(Rho) of the base state
  double *diag_parts = nullptr;  // per-block partials of the statistics
  double *diag_out = nullptr;    // finished statistics
  double2 *diag_spec = nullptr;  // FP64 half spectrum for the energy spectrum
  double *diag_emode = nullptr;  // energy per half-spectrum mode
  int32_t *diag_modes = nullptr;        // mode indices grouped by shell
  int32_t *diag_shell_start = nullptr;  // nshell + 1 offsets into diag_modes
  int diag_nshell = 0;
  double diag_dk = 0;
  int32_t *rdf_counts = nullptr, *rdf_start = nullptr, *rdf_fill = nullptr;
  double *rdf_pos = nullptr;                 // 3np positions grouped by cell
  unsigned long long *rdf_hist = nullptr;
  long long rdf_cells_cap = 0;
  int rdf_bins_cap = 0;

  // ---- profiling ----
  bool prof_on = false;
  std::vector<tpm::ProfEntry> prof;
  std::vector<void *> allocs;
};

namespace tpm {

// launch bookkeeping (tpm_ctx.cu)
void prof_begin(tpm_ctx *c, const char *name, cudaEvent_t *ev0);
void prof_end(tpm_ctx *c, const char *name, cudaEvent_t ev0);

// ---- field kernels (tpm_fields.cu) ----
void launch_p0_update(tpm_ctx *c, int stage);
void launch_rho_update(tpm_ctx *c, int stage, bool np1_in_base);
void launch_face_velocity(tpm_ctx *c);
// the mixed path on grids of whole TMA tiles forms the face velocity in the
// density pass (launch_face_velocity is then a no-op)
bool face_velocity_in_rho_pass(const tpm_ctx *c);
void launch_rhs_momentum(tpm_ctx *c, int stage, bool np1_in_base);
void rhs_kernels_setup(tpm_ctx *c);
void particle_kernels_setup(tpm_ctx *c);  // tpm_particles.cu
void launch_face_coeff(tpm_ctx *c);  // mixed path: C and C/d^2 pairs from Rho_new
void launch_poisson_rhs(tpm_ctx *c, int stage, bool store_div);
void launch_project(tpm_ctx *c, int stage);
void launch_div_residual(tpm_ctx *c, int stage, const double *RUn);
void launch_mean_reset(tpm_ctx *c);
void launch_passive_scalar(tpm_ctx *c, int stage, bool np1_in_base);  // grid.cpp:743-772
void launch_passive_scalar_face(tpm_ctx *c, const double *src);      // PS_face = I_C2F(src)
int cell_blocks(const Grid &g);
// Blocks for a grid-stride kernel over `items` items, `threads` per block:
// whole waves of the blocks the kernel keeps resident (SMs x resident blocks
// per SM from the occupancy calculator, cached per kernel), fewer only when
// the items need fewer.  A reducing kernel (one partial per block) stays
// within kRedBlocks, in whole waves where the SM count allows.
int wave_blocks(tpm_ctx *c, const void *kernel, int threads, long long items, bool reduces);
int zm_blocks(const tpm_ctx *c);  // blocks of the z-marching stencil kernels
int zm_zlen(const tpm_ctx *c);    // their planes per z chunk
void launch_center_coeff_from_C(tpm_ctx *c);  // operator-level Poisson entry
void launch_to_float(tpm_ctx *c, const double *src, float *dst, long long n);
void launch_to_double(tpm_ctx *c, const float *src, double *dst, long long n);

// ---- Poisson / FFT (tpm_fft.cu) ----
void fft_plans_create(tpm_ctx *c);
// A Richardson loop captured as a conditional while node: the body's last
// kernel sets `handle` to continue while it < max_it and max|dp| > epsilon.
struct LoopCtl {
  cudaGraphConditionalHandle handle;
  int max_it;
};
// one Richardson iteration; returns nothing (error lands in dsc->err).  With
// eps_ctl > 0 and no loop control the iteration sets dsc->skip once
// max|dp| <= eps_ctl, and every kernel of a later iteration returns at once.
// One Richardson iteration; the device stops the solve (skip, or the captured
// loop's condition) once max|dp| <= eps_ctl (negative: never).
void poisson_iteration(tpm_ctx *c, double eps_ctl = -1.0, const LoopCtl *loop = nullptr);
// skip = it = 0 and err = 100 (poisson.cpp:395: the error a solve reports
// when it runs no iteration) at the start of a solve
void poisson_loop_begin(tpm_ctx *c);
// mixed Richardson loop: P += dP after the loop (a no-op below two iterations)
void refine_finish(tpm_ctx *c);
// z = S (-Lap_h)^-1 S r, S = diag(sc) (FFT passes of the Poisson solve), with
// per-block partials of r.z; returns the number of partials
int fft_precondition(tpm_ctx *c, const double *r, const double *sc, double *z, double *parts,
                     const int *skip);
void precondition_setup();
// PCG pressure solve (Solver = 2; tpm_pcg.cu): set-up, then one iteration
void pcg_alloc(tpm_ctx *c);
void pcg_setup(tpm_ctx *c, double eps, const LoopCtl *loop);
void pcg_step(tpm_ctx *c, double eps, const LoopCtl *loop);
int pens_default(int n, int elem_bytes);
int pens_max(int n, int elem_bytes);
// energy per half-spectrum mode of the face velocity U3 (3n), summed over
// components (spec: FP64 half-spectrum scratch)
void spectrum_mode_energy(tpm_ctx *c, const double *U3, double2 *spec, double *emode);
void spectrum_kernels_setup();

// ---- step driver (tpm_ctx.cu) and graph replay (tpm_graph.cu) ----
void step_param_update(tpm_ctx *c);  // PARAM.update (params.cpp:80-86)
void step_body(tpm_ctx *c);          // four substeps and the end of step
void step_substep(tpm_ctx *c, int s); // one RK4 stage
void step_end(tpm_ctx *c);           // make_mean_U0 and TimeAdvance
// the pieces of a step whose host transfers overlap it: stage s's head
// (through the push; joins the auxiliary stream at its end) and tail, the
// tail as two parts (through the Poisson solve, whose P is then final; the
// projection, whose RU_int is then final) or as its particle deposits (which
// read neither the step's RU nor P) and the rest, and the end of the step
// without the particle reorder (particle_reorder follows)
void step_stage_head(tpm_ctx *c, int s);
void step_stage_tail(tpm_ctx *c, int s);
void step_stage_tail_solve(tpm_ctx *c, int s);
void step_stage_tail_project(tpm_ctx *c, int s);
void step_stage_tail_deposits(tpm_ctx *c, int s);
void step_stage_tail_rest(tpm_ctx *c, int s);
void step_end_no_reorder(tpm_ctx *c);
// run `body` (one piece of a step, id `piece`) from a graph captured once per
// host state, or eagerly when graphs are off or profiling is on; `advances`:
// the piece ends the step (T_cur and num_timestep move on)
void run_piece(tpm_ctx *c, int piece, bool advances, const std::function<void()> &body);
void step_any(tpm_ctx *c);           // one step, replayed from a graph in graph mode
// tpm_resume without the status wrapper; with rho_ready, the work that reads
// Rho waits for that event (the particle work before it does not)
void resume_device(tpm_ctx *c, cudaEvent_t rho_ready = nullptr);
void graphs_clear(std::vector<GraphEntry> &cache);

// ---- particles (tpm_particles.cu) ----
void launch_particle_push(tpm_ctx *c, int stage, bool np1_in_base);
void particle_deposit_momentum(tpm_ctx *c);
void particle_deposit_concentration(tpm_ctx *c);
void particle_heat(tpm_ctx *c);
void particle_init_heat(tpm_ctx *c);
void particle_resume(tpm_ctx *c);
void particle_zero_fields(tpm_ctx *c);
// mixed path: permute the particles into the cell order of the last heat
// deposit's sort (at a step boundary; pq[2], pq[3] are free there)
void particle_reorder(tpm_ctx *c);
void particles_reorder_init(tpm_ctx *c);  // pid = identity (the caller order)
// per-particle arrays between the caller's order and storage order (elem =
// 8 or 4 bytes); plain copies unless c->reorder
void particles_from_host(tpm_ctx *c, void *dev, const void *host, int elem);
void particles_to_host(tpm_ctx *c, void *host, const void *dev, int elem);
// The particle state (the base set's 7 quantities, then the heat rates) as
// one transfer through kStateArrays staging slots of np doubles: copy_in
// copies the caller's arrays into the slots back to back (directly into the
// base set and rhs_t when the particles keep the caller's order) and
// stage_in permutes the slots into storage with one kernel (from_host: both);
// index forms slot (pid inverted) for the present storage order, after which
// stage_out permutes storage (src, rhs_t) into the slots, and copy_out
// copies the slots to the caller's arrays (directly from src and rhs_t_dev
// when the particles keep the caller's order), each on the current stream.
constexpr int kStateArrays = 8;
void particle_state_copy_in(tpm_ctx *c, const double *const *part, const double *rhs_t);
void particle_state_stage_in(tpm_ctx *c);
void particle_state_from_host(tpm_ctx *c, const double *const *part, const double *rhs_t);
void particle_state_index(tpm_ctx *c);
void particle_state_stage_out(tpm_ctx *c, double *const *src, const double *rhs_t);
void particle_state_copy_out(tpm_ctx *c, double *const *part, double *rhs_t,
                             double *const *src, const double *rhs_t_dev);

}  // namespace tpm

namespace tpm {

// Device allocation owned by the context (freed by tpm_destroy).
template <typename T>
T *dalloc(tpm_ctx *c, size_t count) {
  void *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::make_pair(TPM_ERR_NOMEM, std::string("cudaMalloc of ") +
                                            std::to_string(count * sizeof(T)) + " bytes failed");
  }
  c->allocs.push_back(p);
  return reinterpret_cast<T *>(p);
}

inline int fail(tpm_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

// Runs f, mapping exceptions to status codes (the library never exits).
template <typename F>
int guarded(tpm_ctx *c, F &&f) {
  if (!c) return TPM_ERR_ARG;
  try {
    return f();
  } catch (const std::pair<int, std::string> &e) {
    return fail(c, e.first, e.second);
  } catch (const std::string &s) {
    return fail(c, TPM_ERR_CUDA, s);
  } catch (const std::bad_alloc &) {
    return fail(c, TPM_ERR_NOMEM, "host allocation failed");
  }
}

}  // namespace tpm

#define TPM_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      throw std::string(#expr) + ": " + cudaGetErrorString(e_);              \
    }                                                                        \
  } while (0)

// Launch with bookkeeping: counts launches, optionally times them.
#define TPM_LAUNCH(ctx, name, kernel, grid, block, smem, ...)                \
  do {                                                                       \
    cudaEvent_t ev0_ = nullptr;                                              \
    if ((ctx)->prof_on) tpm::prof_begin((ctx), (name), &ev0_);               \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);         \
    (ctx)->launches++;                                                       \
    TPM_CUDA_TRY(cudaGetLastError());                                        \
    if ((ctx)->prof_on) tpm::prof_end((ctx), (name), ev0_);                  \
  } while (0)
