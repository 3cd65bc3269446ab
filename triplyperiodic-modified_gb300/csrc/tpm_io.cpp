// Restart and dump files in the reference's byte formats, so that a GPU run
// can be continued by the reference build (Initial=1) and a reference run by
// the GPU library.
//
//  * restart set read by grid::Initialize with Initial=1 (grid.cpp:221-238)
//    and particle::Load_All (particle.cpp:939-989): Restart_RU.bin (x, y, z
//    blocks), Restart_Rho.bin, Restart_P.bin - raw native FP64, C order
//    [Nz][Ny][Nx] (communicator.cpp:114-134); Restart_Part_{x,y,z,u,v,w,T}.bin
//    FP64 [Np] and Restart_Part_flag.bin int32 [Np]; Restart_numbers.dat with
//    "P0 T_cur num_timestep" (written here with 17 significant digits); with
//    solve_for_scalar also Restart_Passive_Scalar.bin (Initial_C = 1,
//    grid.cpp:445-450).
//  * dumps written by grid::Store (grid.cpp:525-592) and particle::Store_All
//    (particle.cpp:848-897): RU_<n>.bin, Rho_<n>.bin, P_<n>.bin, Passive_Scalar_<n>.bin,
//    Part_{x,...,flag}_<n>.bin and numbers_<n>.dat, n = num_timestep.
#include <cstdio>
#include <string>
#include <vector>

#include "tpm_internal.cuh"

namespace {

std::string join(const char *dir, const std::string &name) {
  std::string d = dir ? dir : ".";
  if (!d.empty() && d.back() != '/') d += '/';
  return d + name;
}

int io_fail(tpm_ctx *ctx, const std::string &path, const char *what) {
  ctx->err = path + ": " + what;
  return TPM_ERR_ARG;
}

template <typename T>
int write_raw(tpm_ctx *ctx, const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return io_fail(ctx, path, "cannot open for writing");
  size_t n = v.empty() ? 0 : std::fwrite(v.data(), sizeof(T), v.size(), f);
  int rc = std::fclose(f);
  return (n == v.size() && rc == 0) ? TPM_OK : io_fail(ctx, path, "short write");
}

// Reads exactly v.size() elements; a file of any other length is refused, so a
// set written for another grid or particle count never reaches the device.
template <typename T>
int read_raw(tpm_ctx *ctx, const std::string &path, std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return io_fail(ctx, path, "cannot open");
  std::fseek(f, 0, SEEK_END);
  long bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (bytes < 0 || (size_t)bytes != v.size() * sizeof(T)) {
    std::fclose(f);
    return io_fail(ctx, path, ("holds " + std::to_string(bytes) + " bytes, expected " +
                               std::to_string(v.size() * sizeof(T))).c_str());
  }
  size_t n = v.empty() ? 0 : std::fread(v.data(), sizeof(T), v.size(), f);
  std::fclose(f);
  return n == v.size() ? TPM_OK : io_fail(ctx, path, "short read");
}

struct Host {
  std::vector<double> RU, Rho, P, PS;
  std::vector<double> q[7];
  std::vector<int32_t> flag;
};

int download_all(tpm_ctx *ctx, long long n, int64_t np, Host &h) {
  h.RU.resize(3 * n);
  h.Rho.resize(n);
  h.P.resize(n);
  int rc;
  if ((rc = tpm_download_field(ctx, TPM_FIELD_RU, h.RU.data()))) return rc;
  if ((rc = tpm_download_field(ctx, TPM_FIELD_RHO, h.Rho.data()))) return rc;
  if ((rc = tpm_download_field(ctx, TPM_FIELD_P, h.P.data()))) return rc;
  if (ctx->PS) {
    h.PS.resize(n);
    if ((rc = tpm_download_field(ctx, TPM_FIELD_PASSIVE_SCALAR, h.PS.data()))) return rc;
  }
  for (auto &v : h.q) v.resize(np);
  h.flag.resize(np);
  if (np > 0)
    rc = tpm_download_particles(ctx, TPM_PSET_BASE, h.q[0].data(), h.q[1].data(), h.q[2].data(),
                                h.q[3].data(), h.q[4].data(), h.q[5].data(), h.q[6].data(),
                                h.flag.data());
  return rc;
}

const char *kQ[7] = {"x", "y", "z", "u", "v", "w", "T"};

}  // namespace

extern "C" {

int tpm_write_restart(tpm_ctx *ctx, const char *dir) {
  if (!ctx || !dir) return TPM_ERR_ARG;
  const long long n = ctx->g.n;
  const int64_t np = ctx->np;
  Host h;
  int rc = download_all(ctx, n, np, h);
  if (rc) return rc;
  tpm_scalars sc;
  if ((rc = tpm_get_scalars(ctx, &sc)) && rc != TPM_ERR_NONFINITE) return rc;
  if ((rc = write_raw(ctx, join(dir, "Restart_RU.bin"), h.RU))) return rc;
  if ((rc = write_raw(ctx, join(dir, "Restart_Rho.bin"), h.Rho))) return rc;
  if ((rc = write_raw(ctx, join(dir, "Restart_P.bin"), h.P))) return rc;
  if (ctx->PS && (rc = write_raw(ctx, join(dir, "Restart_Passive_Scalar.bin"), h.PS))) return rc;
  for (int q = 0; q < 7; ++q)
    if ((rc = write_raw(ctx, join(dir, std::string("Restart_Part_") + kQ[q] + ".bin"), h.q[q])))
      return rc;
  if ((rc = write_raw(ctx, join(dir, "Restart_Part_flag.bin"), h.flag))) return rc;
  const std::string nf = join(dir, "Restart_numbers.dat");
  FILE *f = std::fopen(nf.c_str(), "w");
  if (!f) return io_fail(ctx, nf, "cannot open for writing");
  std::fprintf(f, "%.17g %.17g %lld\n", sc.P0, sc.T_cur, (long long)sc.num_timestep);
  return std::fclose(f) == 0 ? TPM_OK : io_fail(ctx, nf, "short write");
}

int tpm_read_restart(tpm_ctx *ctx, const char *dir) {
  if (!ctx || !dir) return TPM_ERR_ARG;
  const long long n = ctx->g.n;
  const int64_t np = ctx->np;
  Host h;
  h.RU.resize(3 * n);
  h.Rho.resize(n);
  h.P.resize(n);
  int rc;
  if ((rc = read_raw(ctx, join(dir, "Restart_RU.bin"), h.RU))) return rc;
  if ((rc = read_raw(ctx, join(dir, "Restart_Rho.bin"), h.Rho))) return rc;
  if ((rc = read_raw(ctx, join(dir, "Restart_P.bin"), h.P))) return rc;
  if (ctx->PS) {  // Initial_C = 1 (grid.cpp:445-450)
    h.PS.resize(n);
    if ((rc = read_raw(ctx, join(dir, "Restart_Passive_Scalar.bin"), h.PS))) return rc;
  }
  for (int q = 0; q < 7; ++q) {
    h.q[q].resize(np);
    if ((rc = read_raw(ctx, join(dir, std::string("Restart_Part_") + kQ[q] + ".bin"), h.q[q])))
      return rc;
  }
  h.flag.resize(np);
  if ((rc = read_raw(ctx, join(dir, "Restart_Part_flag.bin"), h.flag))) return rc;
  double P0 = 0, T_cur = 0;
  long long step = 0;
  const std::string nf = join(dir, "Restart_numbers.dat");
  FILE *f = std::fopen(nf.c_str(), "r");
  if (!f) return io_fail(ctx, nf, "cannot open");
  int got = std::fscanf(f, "%lf %lf %lld", &P0, &T_cur, &step);
  std::fclose(f);
  if (got != 3) return io_fail(ctx, nf, "expected \"P0 T_cur num_timestep\"");
  if ((rc = tpm_upload_field(ctx, TPM_FIELD_RU, h.RU.data()))) return rc;
  if ((rc = tpm_upload_field(ctx, TPM_FIELD_RHO, h.Rho.data()))) return rc;
  if ((rc = tpm_upload_field(ctx, TPM_FIELD_P, h.P.data()))) return rc;
  if (ctx->PS && (rc = tpm_upload_field(ctx, TPM_FIELD_PASSIVE_SCALAR, h.PS.data()))) return rc;
  if (np > 0 &&
      (rc = tpm_upload_particles(ctx, TPM_PSET_BASE, h.q[0].data(), h.q[1].data(), h.q[2].data(),
                                 h.q[3].data(), h.q[4].data(), h.q[5].data(), h.q[6].data(),
                                 h.flag.data())))
    return rc;
  return tpm_set_scalars(ctx, P0, T_cur, step);
}

int tpm_store(tpm_ctx *ctx, const char *dir) {
  if (!ctx || !dir) return TPM_ERR_ARG;
  const long long n = ctx->g.n;
  const int64_t np = ctx->np;
  Host h;
  int rc = download_all(ctx, n, np, h);
  if (rc) return rc;
  tpm_scalars sc;
  if ((rc = tpm_get_scalars(ctx, &sc)) && rc != TPM_ERR_NONFINITE) return rc;
  const std::string s = "_" + std::to_string((long long)sc.num_timestep);
  if ((rc = write_raw(ctx, join(dir, "RU" + s + ".bin"), h.RU))) return rc;
  if ((rc = write_raw(ctx, join(dir, "Rho" + s + ".bin"), h.Rho))) return rc;
  if ((rc = write_raw(ctx, join(dir, "P" + s + ".bin"), h.P))) return rc;
  if (ctx->PS && (rc = write_raw(ctx, join(dir, "Passive_Scalar" + s + ".bin"), h.PS))) return rc;
  for (int q = 0; q < 7; ++q)
    if ((rc = write_raw(ctx, join(dir, std::string("Part_") + kQ[q] + s + ".bin"), h.q[q]))) return rc;
  if ((rc = write_raw(ctx, join(dir, "Part_flag" + s + ".bin"), h.flag))) return rc;
  const std::string nf = join(dir, "numbers" + s + ".dat");
  FILE *f = std::fopen(nf.c_str(), "w");
  if (!f) return io_fail(ctx, nf, "cannot open for writing");
  std::fprintf(f, "%.17g\n%.17g\n%lld\n", sc.P0, sc.T_cur, (long long)sc.num_timestep);
  return std::fclose(f) == 0 ? TPM_OK : io_fail(ctx, nf, "short write");
}

}  // extern "C"
