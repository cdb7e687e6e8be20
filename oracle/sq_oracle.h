/*
 * sq_oracle.h -- C ABI of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle restates, in plain FP64 C++, the
 * reference SQMiniApp per-node Spectral Quadrature path (input decks, setup,
 * truncated-cube Hamiltonian, Lanczos, implicit QL).  Only the test suite,
 * __graft_entry__.smoke() and the CPU-baseline legs of bench.py may load it;
 * the product library never links or calls it.
 *
 * Parity status: the reference writes no lambda/weight/density values and
 * cannot be built without PETSc and MPI, so the oracle's numeric outputs are
 * "parity unpinned" against reference outputs.  The oracle is pinned instead
 * by (a) the node and overlap counts that the reference's own run logs print
 * (test/a1.out, a2.out, a4.out, a4a.out) and (b) independent mathematical
 * known-answer tests (dense eigensolves, not-a-knot splines, analytic FD
 * weights and spherical harmonics) in tests/.
 */
#ifndef SQ_ORACLE_H
#define SQ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Open a deck <dir>/<name>.inpt/.ion/.relax with its pseudopotential files in
 * <dir>/pseudopotential/.  faithful=1 keeps the reference's operator quirks
 * (one shared projector coefficient per atom, image range taken from the
 * pseudocharge cutoff, no images for BOUNDARY_CONDITION 2); faithful=0 uses
 * the corrected operator (one coefficient per (atom,l,m), image range from
 * Rcut plus the projector radius, images for every periodic BC).
 * Returns NULL on error and writes a message into err. */
void *sqo_open(const char *dir, const char *name, int faithful, char *err, int errlen);
void sqo_close(void *h);

/* ints[0..15]: nx ny nz, nx_loc ny_loc nz_loc, n_qp, n_nodes, ntype, natoms,
 *              n_images, fd_half_order, bc, n_lm(type 0), total valence electrons, faithful
 * dbls[0..15]: hx hy hz, Rx Ry Rz, Rcut, beta, dV, veff placeholder (0.333), */
int sqo_dims(void *h, int *ints, double *dbls);

/* FD coefficients of -1/2 Laplacian, [0..o] for x, y and z. */
int sqo_fd_coeffs(void *h, double *cx, double *cy, double *cz);

/* Nonlocal coefficients Gamma_l of type t (4 entries, 0 for the local l). */
int sqo_gamma(void *h, int type, double *gamma4);

/* Pseudocharge cutoff (x,y,z) of every type: out[3*ntype]. */
int sqo_pseudocharge_cutoff(void *h, double *out);

/* Radial tables of type t as read from its psd file (r, V_loc, valence density
 * rho_atom = value / (4 pi r^2); each *n entries, any may be NULL) and its valence charge. */
int sqo_psd_tables(void *h, int type, int *n, double *r, double *vloc, double *rho_atom,
                   double *zval);

/* Atom positions pos[natoms][3] and types[natoms] in .ion order. */
int sqo_atoms(void *h, double *pos, int *types);

/* Number of (atom, periodic image) pairs whose pseudocharge box overlaps the
 * block [xcor,xcor+lx) x [ycor,..) x [zcor,..) (GetInfluencingAtoms_Local).
 * If extra_xyz is not NULL an additional atom at that position is included,
 * which models the reference's atom loop running one entry past the end. */
int sqo_local_overlap_count(void *h, int xcor, int ycor, int zcor, int lx, int ly, int lz,
                            const double *extra_xyz, int *count);

/* Per-node Lanczos + quadrature for nodes[0..nsel) (linear node index, x fastest).
 * veff: NULL for a constant veff_const on every cube point, else an array over
 * the nx*ny*nz grid that is wrapped periodically into each cube.
 * a,b: [nsel][n_qp+1] (may be NULL); lambda,w: [nsel][n_qp]; lmin,lmax: [nsel]. */
int sqo_nodes_and_weights(void *h, const double *veff, double veff_const, const long *nodes,
                          long nsel, int nthreads, double *a, double *b, double *lambda,
                          double *w, double *lmin, double *lmax);

/* y = H x on one node's truncated cube (x, y of length nx_loc*ny_loc*nz_loc). */
int sqo_matvec(void *h, const double *veff, double veff_const, long node, const double *x,
               double *y);

/* Implicit QL of one tridiagonal (diag[0..n), sub[0..n), sub[n-1] ignored). */
int sqo_ql(const double *diag, const double *sub, int n, double *lambda, double *w,
           double *lmin, double *lmax);

/* Fermi level by bisection and the node densities / energies (FP64).
 * rho[n_nodes] = (2/dV) sum_q w f;  e_band = 2 sum w lambda f;
 * ts = (2/beta) sum w [f ln f + (1-f) ln(1-f)]  (the -TS term, <= 0). */
int sqo_fermi_density_energy(const double *lambda, const double *w, long n_nodes, int n_qp,
                             double beta, double n_electrons, double dV, double tol,
                             int maxit, double *lambda_f, double *rho, double *e_band,
                             double *ts, int *iters);

/* Cubic spline of the reference (getYD_gen + SplineEvaluate) for tests. */
int sqo_spline(const double *x, const double *y, int n, const double *xq, double *yq, int nq);

/* Real spherical harmonic of the reference for tests. */
double sqo_ylm(double x, double y, double z, int l, int m);

#ifdef __cplusplus
}
#endif
#endif
