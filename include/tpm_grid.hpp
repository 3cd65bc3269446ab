/*
 * tpm_grid.hpp - the reference's grid class (grid.h:14-137) as a header-only
 * C++ facade over libtpm.so (include/tpm.h), so that a time loop written for
 * the reference (simulation.cpp:57-93) keeps its shape:
 *
 *   tpmgpu::grid GRID(params, np);            // grid::grid + PARAM
 *   GRID.Read_Restart(dir);                   // the Initial=1 inputs (grid.cpp:221-238)
 *   GRID.Initialize();                        // grid.cpp:461-484
 *   do {
 *     GRID.param_update();                    // PARAM.update(GRID.T_cur)
 *     for (GRID.RK4_count = 0; GRID.RK4_count < 4; GRID.RK4_count++) {
 *       GRID.Update_Rho();  GRID.Update_P0();  GRID.Update_Particle();
 *       GRID.Update_RU_WOP();  GRID.Compute_Div_U_new();  GRID.Compute_RHS_Pois();
 *       GRID.Solve_Poisson();  GRID.Update_RU_WP();  GRID.TimeAdvance_RK4();
 *     }
 *     GRID.RU_np1_make_mean_U0();              // GRID.RU_np1.make_mean_U0(RhoU_)
 *     GRID.TimeAdvance();
 *     GRID.Statistics();
 *   } while (GRID.T_cur() < T_final);
 *
 * Where the reference's methods return void and print or exit on trouble,
 * these throw tpmgpu::error carrying the library's status and message.  The
 * fields live on the GPU; download() / upload() move them in the reference's
 * file layout ([Nz][Ny][Nx], x fastest; vectors as x, y, z blocks).
 */
#ifndef TPM_GRID_HPP
#define TPM_GRID_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "tpm.h"

namespace tpmgpu {

class error : public std::runtime_error {
 public:
  error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

class grid {
 public:
  int RK4_count = 0;  // grid.h:109

  grid(const tpm_params &params, int64_t np) : nx_(params.Nx), ny_(params.Ny), nz_(params.Nz) {
    const int rc = tpm_create(&params, np, &ctx_);
    if (rc != TPM_OK) {
      const std::string msg = ctx_ ? tpm_last_error(ctx_) : "tpm_create failed";
      tpm_destroy(ctx_);
      ctx_ = nullptr;
      throw error(rc, msg);
    }
  }
  ~grid() { tpm_destroy(ctx_); }
  grid(const grid &) = delete;  // one context owns the box (the reference's grid is not copyable either)
  grid &operator=(const grid &) = delete;

  tpm_ctx *context() const { return ctx_; }

  // ---- the substep (grid.h:112-136) ----
  void Initialize() { check(tpm_initialize(ctx_)); }
  void param_update() { check(tpm_param_update(ctx_)); }
  void Update_Rho() { check(tpm_update_rho(ctx_, RK4_count)); }
  void Update_P0() { check(tpm_update_p0(ctx_, RK4_count)); }
  void Update_Particle() { check(tpm_update_particle(ctx_, RK4_count)); }
  void Update_Passive_Scalar() { check(tpm_update_passive_scalar(ctx_, RK4_count)); }
  void Update_RU_WOP() { check(tpm_update_ru_wop(ctx_, RK4_count)); }
  void Compute_Div_U_new() { check(tpm_compute_div_u_new(ctx_, RK4_count)); }
  void Compute_RHS_Pois() { check(tpm_compute_rhs_pois(ctx_, RK4_count)); }
  void Solve_Poisson() { check(tpm_solve_poisson(ctx_, RK4_count)); }
  void Update_RU_WP() { check(tpm_update_ru_wp(ctx_, RK4_count)); }
  void TimeAdvance_RK4() { check(tpm_time_advance_rk4(ctx_, RK4_count)); }
  void RU_np1_make_mean_U0() { check(tpm_make_mean_u0(ctx_)); }
  void TimeAdvance() { check(tpm_time_advance(ctx_)); }

  // ---- whole steps (the fused path: independent kernels side by side) ----
  void step() { check(tpm_step(ctx_)); }
  void run(int nsteps) { check(tpm_run(ctx_, nsteps)); }
  void sync() { check(tpm_sync(ctx_)); }

  // ---- statistics and files (grid.cpp:902-940, 221-238, 525-592) ----
  tpm_stats Statistics() {
    tpm_stats s;
    check(tpm_statistics(ctx_, &s));
    return s;
  }
  void Read_Restart(const std::string &dir) { check(tpm_read_restart(ctx_, dir.c_str())); }
  void Write_Restart(const std::string &dir) { check(tpm_write_restart(ctx_, dir.c_str())); }
  void Store(const std::string &dir) { check(tpm_store(ctx_, dir.c_str())); }

  // ---- state ----
  tpm_scalars scalars() {
    tpm_scalars s;
    check(tpm_get_scalars(ctx_, &s));
    return s;
  }
  double T_cur() { return scalars().T_cur; }
  int64_t num_timestep() { return scalars().num_timestep; }
  std::vector<double> download(int field) {
    std::vector<double> v(field_len(field));
    check(tpm_download_field(ctx_, field, v.data()));
    return v;
  }
  void upload(int field, const std::vector<double> &v) {
    if (v.size() != field_len(field)) throw error(TPM_ERR_ARG, "field size");
    check(tpm_upload_field(ctx_, field, v.data()));
  }

 private:
  void check(int rc) const {
    if (rc != TPM_OK) throw error(rc, tpm_last_error(ctx_));
  }
  size_t field_len(int field) const {
    const size_t n = (size_t)nx_ * ny_ * nz_;
    const bool vec = field == TPM_FIELD_RU || field == TPM_FIELD_RU_INT || field == TPM_FIELD_RU_NEW ||
                     field == TPM_FIELD_RU_NP1 || field == TPM_FIELD_FP;
    return vec ? 3 * n : n;
  }

  tpm_ctx *ctx_ = nullptr;
  int nx_, ny_, nz_;
};

}  // namespace tpmgpu

#endif  // TPM_GRID_HPP
