// Driver for the reference solver's own sources (test infrastructure).
//
// It replaces simulation.cpp's main (simulation.cpp:16-108) so that the
// reference can be run for an exact number of RK4 steps and its state dumped
// for parity checks.  The loop body is the reference's time loop
// (simulation.cpp:57-93) with one deliberate difference: the particle stage
// `GRID.Update_Particle()` that is commented out at simulation.cpp:64 is
// called, so that two-way coupling and particle heating are active.  Passing
// `--as-shipped` skips it and reproduces the shipped loop.
//
// usage: tpm_ref <deck> <nsteps> <outdir> [--as-shipped] [--substeps S] [--stats]
//   Run in a directory holding the Restart_* files the deck's Initial=1 reads
//   (grid.cpp:221-238, particle.cpp:939-989).  With --substeps S (1..4) only
//   the first S RK4 substeps of the first step run and no end-of-step work is
//   done, for substep-level comparisons.  With --stats grid::Statistics runs
//   after each step, as at simulation.cpp:92 (the deck must set Statistics=1;
//   it appends to <Stat_dir>/<name>.dat).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <mpi.h>

#include "communicator.h"
#include "grid.h"
#include "gridsize.h"
#include "params.h"
#include "poisson.h"
#include "proc.h"
#include "tensor0.h"
#include "tensor1.h"

template <typename T>
static void dump_vec(const std::string &path, const std::vector<T> &v, int n) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (n > 0) std::fwrite(v.data(), sizeof(T), (size_t)n, f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s deck nsteps outdir [--as-shipped] [--substeps S]\n", argv[0]);
    return 1;
  }
  int nsteps = std::atoi(argv[2]);
  std::string out = argv[3];
  bool as_shipped = false, stats = false;
  int substeps = 0;
  for (int a = 4; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--as-shipped")) as_shipped = true;
    else if (!std::strcmp(argv[a], "--stats")) stats = true;
    else if (!std::strcmp(argv[a], "--substeps") && a + 1 < argc) substeps = std::atoi(argv[++a]);
  }
  MPI_Init(&argc, &argv);
  params PARAM(argv[1]);
  double RhoU_[3] = {PARAM.U0() * PARAM.Rho0(), PARAM.V0() * PARAM.Rho0(), PARAM.W0() * PARAM.Rho0()};
  proc PROC;
  gridsize GSIZE(&PARAM, &PROC);
  communicator COMM(&GSIZE, &PARAM, &PROC);
  // The grid object is never destroyed: its destructor would free the
  // uninitialised dQ member (grid.cpp:12 initialiser list omits it).
  grid *G = new grid(&GSIZE, &PARAM, &PROC, &COMM);
  grid &GRID = *G;
  GRID.Initialize();

  auto t0 = std::chrono::steady_clock::now();
  int done = 0;
  if (substeps > 0) {
    PARAM.update(GRID.T_cur);
    for (GRID.RK4_count = 0; GRID.RK4_count < substeps; GRID.RK4_count++) {
      GRID.Update_Rho();
      GRID.Update_P0();
      if (!as_shipped) GRID.Update_Particle();
      if (PARAM.solve_for_scalar()) GRID.Update_Passive_Scalar();  // simulation.cpp:65
      GRID.Update_RU_WOP();
      GRID.Compute_Div_U_new();
      GRID.Compute_RHS_Pois();
      GRID.Solve_Poisson();
      GRID.Update_RU_WP();
      GRID.TimeAdvance_RK4();
    }
  } else {
    for (done = 0; done < nsteps; ++done) {
      PARAM.update(GRID.T_cur);
      for (GRID.RK4_count = 0; GRID.RK4_count < 4; GRID.RK4_count++) {
        GRID.Update_Rho();
        GRID.Update_P0();
        if (!as_shipped) GRID.Update_Particle();
        if (PARAM.solve_for_scalar()) GRID.Update_Passive_Scalar();  // simulation.cpp:65
        GRID.Update_RU_WOP();
        GRID.Compute_Div_U_new();
        GRID.Compute_RHS_Pois();
        GRID.Solve_Poisson();
        GRID.Update_RU_WP();
        GRID.TimeAdvance_RK4();
      }
      GRID.RU_np1.make_mean_U0(RhoU_);
      GRID.TimeAdvance();
      if (stats) GRID.Statistics();
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  double secs = std::chrono::duration<double>(t1 - t0).count();

  // ---- dumps: fields in the reference's global x-fastest layout ----
  auto P = [&](const char *name) { return out + "/" + name; };
  COMM.write(GRID.RU, (char *)P("RU.bin").c_str());
  COMM.write(GRID.RU_int, (char *)P("RU_int.bin").c_str());
  COMM.write(GRID.RU_np1, (char *)P("RU_np1.bin").c_str());
  COMM.write(GRID.RU_new, (char *)P("RU_new.bin").c_str());
  COMM.write(GRID.Rho, (char *)P("Rho.bin").c_str());
  COMM.write(GRID.Rho_new, (char *)P("Rho_new.bin").c_str());
  COMM.write(GRID.Rho_np1, (char *)P("Rho_np1.bin").c_str());
  COMM.write(GRID.P, (char *)P("P.bin").c_str());
  COMM.write(GRID.C, (char *)P("C.bin").c_str());
  COMM.write(GRID.RHS_Part_Temp, (char *)P("RHS_Part_Temp.bin").c_str());
  COMM.write(GRID.RHS_RU, (char *)P("RHS_RU.bin").c_str());
  COMM.write(GRID.RHS_Pois, (char *)P("RHS_Pois.bin").c_str());
  COMM.write(GRID.divergence, (char *)P("divergence.bin").c_str());
  if (PARAM.solve_for_scalar())
    COMM.write(GRID.Passive_Scalar, (char *)P("Passive_Scalar.bin").c_str());
  int np = GRID.part.Np;
  dump_vec(P("Part_x.bin"), GRID.part.x, np);
  dump_vec(P("Part_y.bin"), GRID.part.y, np);
  dump_vec(P("Part_z.bin"), GRID.part.z, np);
  dump_vec(P("Part_u.bin"), GRID.part.u, np);
  dump_vec(P("Part_v.bin"), GRID.part.v, np);
  dump_vec(P("Part_w.bin"), GRID.part.w, np);
  dump_vec(P("Part_T.bin"), GRID.part.T, np);
  dump_vec(P("Part_flag.bin"), GRID.part.flag, np);
  dump_vec(P("Part_RHS_T.bin"), GRID.part.RHS_T, np);
  dump_vec(P("Part_x_np1.bin"), GRID.part.x_np1, np);
  dump_vec(P("Part_y_np1.bin"), GRID.part.y_np1, np);
  dump_vec(P("Part_z_np1.bin"), GRID.part.z_np1, np);
  dump_vec(P("Part_u_np1.bin"), GRID.part.u_np1, np);
  dump_vec(P("Part_v_np1.bin"), GRID.part.v_np1, np);
  dump_vec(P("Part_w_np1.bin"), GRID.part.w_np1, np);
  dump_vec(P("Part_T_np1.bin"), GRID.part.T_np1, np);
  dump_vec(P("Part_x_int.bin"), GRID.part.x_int, np);
  dump_vec(P("Part_y_int.bin"), GRID.part.y_int, np);
  dump_vec(P("Part_z_int.bin"), GRID.part.z_int, np);
  dump_vec(P("Part_u_int.bin"), GRID.part.u_int, np);
  dump_vec(P("Part_v_int.bin"), GRID.part.v_int, np);
  dump_vec(P("Part_w_int.bin"), GRID.part.w_int, np);
  dump_vec(P("Part_T_int.bin"), GRID.part.T_int, np);
  FILE *f = std::fopen(P("scalars.txt").c_str(), "w");
  std::fprintf(f, "%.17g %.17g %.17g %.17g %d %d %d %.17g\n", GRID.P0, GRID.P0_np1, GRID.P0_int,
               GRID.T_cur, GRID.num_timestep, np, done, secs);
  std::fclose(f);
  std::printf("{\"steps\": %d, \"substeps\": %d, \"seconds\": %.6f, \"np\": %d}\n", done, substeps,
              secs, np);
  std::fflush(stdout);
  std::_Exit(0);
}
