// driver.cpp -- sq_lsdft, the command-line program of the engine: the counterpart of the
// reference's main (src/main.cc:19-74) over the C ABI of sq_gb300.h.
//
// The reference runs Get_Input, Initialize, the influencing-atom and projector setup
// (main.cc:32-44), then NodesAndWeights_LSSGQ (main.cc:54) and prints the time spent in SQ and
// in total.  sq_lsdft does the same for one GPU: sq_create_from_deck is the setup,
// sq_nodes_and_weights the SQ pass (Veff = the reference's 0.333 placeholder, scf.cc:71).
// Options add what the reference declares but does not run: the SCF (SCF_LSSGQ, lsdft.h:153),
// the .lambdas and .den files (Print_MinMaxLambda / Print_ElecDens,
// lsdft_readfiles.cc:1106-1138,1294-1381) and the .out echo (:520-607).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sq_gb300.h"

namespace {

const char *kUsage =
    "usage: sq_lsdft -name NAME [-dir DIR] [-precision 32|64] [-faithful 0|1] [-device N]\n"
    "                [-scf] [-lambdas PREFIX] [-den PREFIX] [-out PATH]\n"
    "  reads DIR/NAME.inpt, .ion, .relax and DIR/pseudopotential/<psd>; runs the SQ pass\n"
    "  (and with -scf the SCF loop) on one GPU\n";

double now() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

int fail(const char *what) {
  std::fprintf(stderr, "sq_lsdft: %s: %s\n", what, sq_last_error_string());
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  std::string name, dir = ".", lambdas, den, out;
  sq_options opt = {0, 32, 0, 0, 0, 0};
  bool scf = false;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    const bool has_value = i + 1 < argc;
    if (a == "-name" && has_value) name = argv[++i];
    else if (a == "-dir" && has_value) dir = argv[++i];
    else if (a == "-precision" && has_value) opt.precision = std::atoi(argv[++i]);
    else if (a == "-faithful" && has_value) opt.faithful = std::atoi(argv[++i]);
    else if (a == "-device" && has_value) opt.device = std::atoi(argv[++i]);
    else if (a == "-lambdas" && has_value) lambdas = argv[++i];
    else if (a == "-den" && has_value) den = argv[++i];
    else if (a == "-out" && has_value) out = argv[++i];
    else if (a == "-scf") scf = true;
    else {
      std::fputs(kUsage, stderr);
      return 2;
    }
  }
  if (name.empty()) {
    std::fputs(kUsage, stderr);
    return 2;
  }

  const double t0 = now();
  sq_handle *h = nullptr;
  if (sq_create_from_deck(dir.c_str(), name.c_str(), &opt, &h) != SQ_OK) return fail("setup");
  sq_info info;
  sq_get_info(h, &info);
  std::printf("setup: %d atoms, %d atom images, grid %d x %d x %d (%ld nodes), cube %d^3, "
              "%d Lanczos steps, FP%d, %s operator\n",
              info.n_atoms, info.n_images, info.grid[0], info.grid[1], info.grid[2], info.n_nodes,
              info.cube[0], info.n_qp, opt.precision, opt.faithful ? "reference" : "corrected");
  if (out.empty()) out = dir + "/" + name + ".out";
  if (sq_write_output_echo(h, out.c_str()) != SQ_OK) {
    const int rc = fail("output echo");
    sq_destroy(h);
    return rc;
  }

  const long n = info.n_nodes;
  std::vector<double> lam((size_t)n * info.n_qp), w(lam.size()), lmin(n), lmax(n);
  const double t1 = now();
  if (sq_nodes_and_weights(h, nullptr, 0.333, 0, n, lam.data(), w.data(), lmin.data(),
                           lmax.data()) != SQ_OK) {
    const int rc = fail("SQ pass");
    sq_destroy(h);
    return rc;
  }
  const double t2 = now();
  std::printf("Time spent in SQ=%lf s (%.0f node-Lanczos/s)\n", t2 - t1, n / (t2 - t1));
  const int corner[3] = {0, 0, 0};
  if (!lambdas.empty() &&
      sq_write_lambda_file(lambdas.c_str(), 0, corner, info.grid, lmin.data(), lmax.data()) != SQ_OK) {
    const int rc = fail("lambda file");
    sq_destroy(h);
    return rc;
  }

  if (scf) {
    sq_scf_options so;
    std::memset(&so, 0, sizeof(so));  // zeros: the deck's TOL_SCF, MAXIT_SCF and mixing
    sq_scf_result r;
    const sq_status st = sq_scf_run(h, &so, nullptr, &r);
    if (st != SQ_OK && st != SQ_NO_CONVERGENCE) {
      const int rc = fail("SCF");
      sq_destroy(h);
      return rc;
    }
    std::printf("SCF %s after %d iterations: free energy %.10f Ha (%.10f Ha/atom), Fermi level "
                "%.10f Ha, residual %.3e (tol %.1e), %.3f s\n",
                r.converged ? "converged" : "NOT converged", r.iterations, r.free_energy,
                r.free_energy_per_atom, r.lambda_f, r.residual, r.tol, r.seconds);
    if (!den.empty()) {
      std::vector<double> rho(n), rho_next(n);
      if (sq_scf_get_density(h, rho.data(), rho_next.data()) != SQ_OK ||
          sq_write_density_file(den.c_str(), 0, corner, info.grid, rho.data()) != SQ_OK) {
        const int rc = fail("density file");
        sq_destroy(h);
        return rc;
      }
    }
    if (st == SQ_NO_CONVERGENCE) {
      sq_destroy(h);
      return 3;
    }
  }
  std::printf("Total time spent=%lf s\n", now() - t0);
  sq_destroy(h);
  return 0;
}
