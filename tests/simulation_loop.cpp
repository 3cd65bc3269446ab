// The reference's time loop (simulation.cpp:57-93, with Update_Particle
// enabled) over the GPU grid facade (include/tpm_grid.hpp): a C++ caller
// linked against libtpm.so the way the reference's driver would be.
//
//   simulation_loop <params.bin> <np> <restart_dir> <nsteps> <out_dir>
//
// params.bin holds one tpm_params struct as the caller's deck converter
// wrote it; the run starts from the Initial=1 restart files in restart_dir,
// takes nsteps steps and writes the final restart set to out_dir.  It prints
// one line of grid::Statistics per step.  Before the first stage it checks
// that a method called out of the reference's order is refused.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "tpm_grid.hpp"

int main(int argc, char **argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s params.bin np restart_dir nsteps out_dir\n", argv[0]);
    return 2;
  }
  tpm_params p;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f || std::fread(&p, sizeof(p), 1, f) != 1) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  std::fclose(f);
  const long long np = std::atoll(argv[2]);
  const int nsteps = std::atoi(argv[4]);
  try {
    tpmgpu::grid GRID(p, np);
    GRID.Read_Restart(argv[3]);
    GRID.Initialize();
    try {  // out of order: the projection before the stage's density update
      GRID.Solve_Poisson();
      std::fprintf(stderr, "Solve_Poisson before Update_Rho was accepted\n");
      return 1;
    } catch (const tpmgpu::error &e) {
      if (e.code() != TPM_ERR_STATE) throw;
    }
    for (int n = 0; n < nsteps; ++n) {  // simulation.cpp:57
      GRID.param_update();                // PARAM.update(GRID.T_cur)
      for (GRID.RK4_count = 0; GRID.RK4_count < 4; GRID.RK4_count++) {
        GRID.Update_Rho();
        GRID.Update_P0();
        GRID.Update_Particle();
        if (p.solve_for_scalar) GRID.Update_Passive_Scalar();
        GRID.Update_RU_WOP();
        GRID.Compute_Div_U_new();
        GRID.Compute_RHS_Pois();
        GRID.Solve_Poisson();
        GRID.Update_RU_WP();
        GRID.TimeAdvance_RK4();
      }
      GRID.RU_np1_make_mean_U0();  // GRID.RU_np1.make_mean_U0(RhoU_)
      GRID.TimeAdvance();
      const tpm_stats s = GRID.Statistics();
      std::printf("step %lld T %.17g TKE %.17g P0 %.17g iterations %d\n",
                  (long long)s.num_timestep, s.T_cur, s.TKE, s.P0, s.num_iteration);
    }
    GRID.Write_Restart(argv[5]);
  } catch (const tpmgpu::error &e) {
    std::fprintf(stderr, "tpm error %d: %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
