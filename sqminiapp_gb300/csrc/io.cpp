// io.cpp -- the reference's text files for densities, Lanczos spectral bounds and the output
// echo, so that a run of this engine and a run of the reference can read each other's files.
//
//   <prefix>_<rank>.den      Print_ElecDens / Read_ElecDens (src/lsdft_readfiles.cc:1106-1138,
//                            1242-1289): header "xcor ycor zcor lx ly lz", then one line
//                            "k j i value" (%0.16lf) per point of the block, x fastest.
//   <prefix>_<rank>.lambdas  Print_MinMaxLambda / Read_MinMaxLambda (:1294-1381): the same
//                            header, then "LIpos lambda_min lambda_max" per point.
//   <name>.out               the "Input parameters" / "Initialization" echo of :520-607
//                            for the keywords this engine reads.
// A block is the (corner, dims) of one rank's part of the grid; one GPU owns the whole grid,
// corner (0,0,0) and dims = FD_GRID.  Reading checks the header against the expected block
// ("Different domain decomposition used in density input file" in the reference).
#include <cmath>
#include <cstdio>
#include <ctime>
#include <string>

#include "handle.hpp"
#include "sq_gb300.h"

namespace {

std::string block_file(const char *prefix, int rank, const char *ext) {
  return std::string(prefix) + "_" + std::to_string(rank) + ext;
}

bool bad_block(const int corner[3], const int dims[3]) {
  return !corner || !dims || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || corner[0] < 0 ||
         corner[1] < 0 || corner[2] < 0;
}

struct File {
  FILE *f = nullptr;
  File(const std::string &path, const char *mode) : f(std::fopen(path.c_str(), mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

sq_status read_header(FILE *f, const int corner[3], const int dims[3], const std::string &path) {
  int h[6];
  if (std::fscanf(f, "%d %d %d %d %d %d", &h[0], &h[1], &h[2], &h[3], &h[4], &h[5]) != 6)
    return sq::fail(SQ_BAD_INPUT, path + ": missing block header");
  for (int a = 0; a < 3; a++)
    if (h[a] != corner[a] || h[3 + a] != dims[a])
      return sq::fail(SQ_BAD_INPUT, path + ": different domain decomposition used in the file");
  return SQ_OK;
}

}  // namespace

extern "C" {

sq_status sq_write_density_file(const char *prefix, int rank, const int corner[3],
                                const int dims[3], const double *rho) {
  if (!prefix || !rho || bad_block(corner, dims)) return sq::fail(SQ_BAD_INPUT, "bad argument");
  const std::string path = block_file(prefix, rank, ".den");
  File fl(path, "w");
  if (!fl.f) return sq::fail(SQ_BAD_INPUT, "Couldn't create density file " + path);
  std::fprintf(fl.f, "%d %d %d %d %d %d\n", corner[0], corner[1], corner[2], dims[0], dims[1], dims[2]);
  long long e = 0;
  for (int k = corner[2]; k < corner[2] + dims[2]; k++)
    for (int j = corner[1]; j < corner[1] + dims[1]; j++)
      for (int i = corner[0]; i < corner[0] + dims[0]; i++)
        std::fprintf(fl.f, "%d %d %d %0.16lf\n", k, j, i, rho[e++]);
  if (std::ferror(fl.f)) return sq::fail(SQ_BAD_INPUT, "write error on " + path);
  return SQ_OK;
}

sq_status sq_read_density_file(const char *prefix, int rank, const int corner[3], const int dims[3],
                               double *rho) {
  if (!prefix || !rho || bad_block(corner, dims)) return sq::fail(SQ_BAD_INPUT, "bad argument");
  const std::string path = block_file(prefix, rank, ".den");
  File fl(path, "r");
  if (!fl.f) return sq::fail(SQ_BAD_INPUT, "Couldn't open density file " + path);
  sq_status st = read_header(fl.f, corner, dims, path);
  if (st != SQ_OK) return st;
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  for (long long c = 0; c < n; c++) {
    int K, J, I;
    double v;
    if (std::fscanf(fl.f, "%d %d %d %lf", &K, &J, &I, &v) != 4)
      return sq::fail(SQ_BAD_INPUT, path + ": truncated");
    // the reference stores by the (k,j,i) of each line
    if (K < corner[2] || K >= corner[2] + dims[2] || J < corner[1] || J >= corner[1] + dims[1] ||
        I < corner[0] || I >= corner[0] + dims[0])
      return sq::fail(SQ_BAD_INPUT, path + ": point outside the block");
    rho[((long long)(K - corner[2]) * dims[1] + (J - corner[1])) * dims[0] + (I - corner[0])] = v;
  }
  return SQ_OK;
}

sq_status sq_write_lambda_file(const char *prefix, int rank, const int corner[3], const int dims[3],
                               const double *lambda_min, const double *lambda_max) {
  if (!prefix || !lambda_min || !lambda_max || bad_block(corner, dims))
    return sq::fail(SQ_BAD_INPUT, "bad argument");
  const std::string path = block_file(prefix, rank, ".lambdas");
  File fl(path, "w");
  if (!fl.f) return sq::fail(SQ_BAD_INPUT, "Couldn't create lambda file " + path);
  std::fprintf(fl.f, "%d %d %d %d %d %d\n", corner[0], corner[1], corner[2], dims[0], dims[1], dims[2]);
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  for (long long p = 0; p < n; p++)
    std::fprintf(fl.f, "%lld %0.16lf %0.16lf\n", p, lambda_min[p], lambda_max[p]);
  if (std::ferror(fl.f)) return sq::fail(SQ_BAD_INPUT, "write error on " + path);
  return SQ_OK;
}

sq_status sq_read_lambda_file(const char *prefix, int rank, const int corner[3], const int dims[3],
                              double *lambda_min, double *lambda_max) {
  if (!prefix || !lambda_min || !lambda_max || bad_block(corner, dims))
    return sq::fail(SQ_BAD_INPUT, "bad argument");
  const std::string path = block_file(prefix, rank, ".lambdas");
  File fl(path, "r");
  if (!fl.f) return sq::fail(SQ_BAD_INPUT, "Couldn't open lambda file " + path);
  sq_status st = read_header(fl.f, corner, dims, path);
  if (st != SQ_OK) return st;
  const long long n = (long long)dims[0] * dims[1] * dims[2];
  for (long long c = 0; c < n; c++) {
    long long p;
    double lo, hi;
    if (std::fscanf(fl.f, "%lld %lf %lf", &p, &lo, &hi) != 3)
      return sq::fail(SQ_BAD_INPUT, path + ": truncated");
    if (p < 0 || p >= n) return sq::fail(SQ_BAD_INPUT, path + ": point outside the block");
    lambda_min[p] = lo;
    lambda_max[p] = hi;
  }
  return SQ_OK;
}

sq_status sq_write_output_echo(const sq_handle *h, const char *path) {
  if (!h || !path) return sq::fail(SQ_BAD_INPUT, "null argument");
  File fl(path, "w");
  if (!fl.f) return sq::fail(SQ_BAD_INPUT, std::string("Couldn't create output file ") + path);
  FILE *f = fl.f;
  const sq::Deck &d = h->deck;
  const std::time_t now = std::time(nullptr);
  char when[64];
  std::strftime(when, sizeof(when), "%a %b %d %H:%M:%S %Y", std::localtime(&now));
  const char *rule = "***************************************************************************\n";
  std::fprintf(f, "%s", rule);
  std::fprintf(f, "*        GB300 Spectral Quadrature engine (SQMiniApp input decks)        *\n");
  std::fprintf(f, "*                 Start time: %-24s                    *\n", when);
  std::fprintf(f, "%s", rule);
  std::fprintf(f, "                           Input parameters                                \n");
  std::fprintf(f, "%s", rule);
  std::fprintf(f, "CELL: %f %f %f \n", d.cell_half[0], d.cell_half[1], d.cell_half[2]);
  std::fprintf(f, "FD_GRID: %d %d %d\n", d.grid[0], d.grid[1], d.grid[2]);
  std::fprintf(f, "FD_ORDER: %d\n", 2 * d.half_order);
  std::fprintf(f, "BOUNDARY_CONDITION: %d\n", d.bc);
  std::fprintf(f, "BETA: %lf\n", d.beta);
  std::fprintf(f, "LANCZOS_DEGREE: %d\n", d.n_qp);
  std::fprintf(f, "RADIUS_TRUNC: %lf\n", d.rcut);
  std::fprintf(f, "NTYPE: %d\n", (int)d.psd.size());
  std::fprintf(f, "EXCHANGE_CORRELATION: %s\n", d.xc.c_str());
  std::fprintf(f, "MAXIT_SCF: %d\n", d.maxit_scf);
  std::fprintf(f, "TOL_SCF: %E\n", d.tol_scf);
  std::fprintf(f, "MIXING_PARAMETER: %f\n", d.mixing_parameter);
  std::fprintf(f, "MIXING_HISTORY: %d\n", d.mixing_history);
  std::fprintf(f, "PULAY_FREQUENCY: %d\n", d.pulay_frequency);
  std::fprintf(f, "REFERENCE_CUTOFF: %f\n", d.reference_cutoff);
  std::fprintf(f, "PSEUDOPOTENTIAL_FILE:");
  for (const std::string &p : d.psd_file) std::fprintf(f, " %s", p.c_str());
  std::fprintf(f, "\nPSEUDOPOTENTIAL_LOCAL:");
  for (int l : d.lloc) std::fprintf(f, " %d", l);
  std::fprintf(f, "\n%s", rule);
  std::fprintf(f, "                             Initialization                                \n");
  std::fprintf(f, "%s", rule);
  std::fprintf(f, "Number of GPUs                     :  1\n");
  const double *hh = h->setup.h;
  if (std::fabs(hh[0] - hh[1]) <= 1e-15 && std::fabs(hh[0] - hh[2]) <= 1e-15) {
    std::fprintf(f, "Mesh spacing                       : % E (Bohr)\n", hh[0]);
  } else {
    std::fprintf(f, "Mesh spacing in x-direction        : % E (Bohr)\n", hh[0]);
    std::fprintf(f, "Mesh spacing in y-direction        : % E (Bohr)\n", hh[1]);
    std::fprintf(f, "Mesh spacing in z direction        : % E (Bohr)\n", hh[2]);
  }
  std::fprintf(f, "FD nodes                           :  %ld\n", h->info.n_nodes);
  std::fprintf(f, "Truncated cube                     :  %d x %d x %d\n", h->info.cube[0],
               h->info.cube[1], h->info.cube[2]);
  std::fprintf(f, "Lanczos precision                  :  FP%d\n", h->opt.precision);
  std::fprintf(f, "Output printed to                  :  %s\n", path);
  if (std::ferror(f)) return sq::fail(SQ_BAD_INPUT, std::string("write error on ") + path);
  return SQ_OK;
}

}  // extern "C"
