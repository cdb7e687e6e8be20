/*
 * sq_gb300.h -- C ABI of the GB300 Spectral Quadrature engine.
 *
 * The library replaces the per-node Spectral Quadrature path of SQMiniApp:
 * the truncated-cube Hamiltonian matvec (src/lsdft_matvec.cc), the nonlocal
 * projector setup and apply (src/lsdft_nl.cc), the Lanczos recurrence and the
 * tridiagonal quadrature of src/lsdft_scf.cc:32-164 and
 * src/lsdft_tools.cc:912-1026, and the density / Fermi-level / energy closure
 * that src/lsdft.h:98-102,209 declares.  Everything runs on one GPU; there is
 * no CPU fallback.  All pointers are plain host or device pointers, all sizes
 * are element counts, and every call returns an sq_status.
 *
 * Threading: one handle is single-threaded and stream-ordered; separate
 * handles are independent.  The handle owns its device buffers; the caller
 * owns every buffer it passes in.
 */
#ifndef SQ_GB300_H
#define SQ_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference exit(1)s on every error (src/lsdft_readfiles.cc:141-145,
 * :874-877; src/lsdft_tools.cc:20-26,136-139,950-952); here each one is a return value. */
typedef enum sq_status {
  SQ_OK = 0,
  SQ_BAD_INPUT = 1,          /* unreadable deck, inconsistent sizes, unsupported option */
  SQ_NO_CONVERGENCE = 2,     /* implicit QL needed more than 50 sweeps (tools.cc:950-952) */
  SQ_LANCZOS_BREAKDOWN = 3,  /* b_k == 0: the reference divides by it (scf.cc:131,147) */
  SQ_DEVICE_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  SQ_CUDA_ERROR = 5,         /* a CUDA runtime call failed */
  SQ_CAPACITY = 6            /* a per-node atom list exceeded its on-chip capacity */
} sq_status;

typedef struct sq_handle sq_handle;

/* Engine options. */
typedef struct sq_options {
  /* 1: keep the reference operator exactly, including its quirks: all (l,m) projectors of an
   *    atom share one coefficient (src/lsdft_matvec.cc:97-100,136-138), periodic images come
   *    from the pseudocharge cutoff (src/lsdft_initObjs.cc:1765-1772) and
   *    BOUNDARY_CONDITION 2 adds no images (:1763-1784).
   * 0: corrected operator: one coefficient per (atom,l,m) (src/lsdft_matvec.cc:214-227),
   *    image range from Rcut plus the projector radius, images for every periodic BC. */
  int faithful;
  /* 32: FP32 Lanczos vectors and matvecs, FP64 recurrence coefficients, quadrature and sums.
   * 64: FP64 everywhere. */
  int precision;
  int device;   /* CUDA device ordinal */
  /* Per-node projector list format of the FP32 corrected operator: 0 automatic (compact when
   * the full lists of all SMs would not stay in L2), 1 full (chi_lm and packed P|U indices per
   * point), 2 compact (T_l per channel and box coordinates; chi_lm rebuilt while streaming).
   * FP64 and the faithful operator always use the full format. */
  int list_format;
  /* FP32 Lanczos kernel: 0 automatic (the split-pass kernel where it applies: corrected
   * operator, the full lists in L2, both vectors on one CTA -- or, for larger cubes such as
   * 31^3 and 33^3, on a cluster of two CTAs per node), 1 the single-pass kernel, 2 the
   * split-pass kernel (SQ_BAD_INPUT where it does not apply). */
  int kernel;
  /* Split-pass kernel tile: z-ranges per cube row in the z pass and y-ranges per plane in the
   * y pass (threads = ceil(nx/4) * max(ny,nz) * tile); 0 automatic (the engine's autotuner
   * times the candidates on the first call and keeps the fastest).  The two-CTA form runs
   * one tile and needs 0. */
  int tile;
} sq_options;

/* Engine facts after setup. */
typedef struct sq_info {
  int grid[3];          /* FD nodes per axis (FD_GRID) */
  int cube[3];          /* truncated-cube points per axis, 2*ceil(Rcut/h)+1 (readfiles.cc:442-444) */
  int n_qp;             /* LANCZOS_DEGREE */
  int fd_half_order;    /* FD_ORDER / 2 */
  int bc;               /* BOUNDARY_CONDITION */
  int n_atoms;
  int n_types;
  int n_images;         /* atom images whose projector box meets the extended domain */
  int n_tables;         /* distinct projector tables after periodic deduplication */
  int max_images_per_node;  /* on-chip capacity of the per-node image list */
  int precision;
  int faithful;
  long n_nodes;         /* grid[0]*grid[1]*grid[2] */
  double h[3];          /* mesh spacing */
  double cell_half[3];  /* CELL: half side lengths R */
  double rcut;
  double beta;          /* BETA, 1/Ha */
  double dV;
  double n_electrons;   /* sum of valence electrons from the .ion file */
  int n_lm;             /* nonlocal (l,m) projectors per atom (union over types) */
  double proj_points_per_node;  /* mean over nodes of sum_images |projector box ∩ cube| */
  /* Lanczos kernel configuration (0 from sq_describe_deck): vector layout flags (1 = zero rows
   * between z-planes, FP32; 2 = cubes wider than 32 points, FP32; 4 = rows without zero
   * columns, FP64; 8 = compact projector list; 16 = split-pass kernel over 16-byte quads,
   * FP32; 32 = with 16, a cluster of two CTAs per node, the cube split in z), U on chip (1) or
   * in global scratch (0), threads per CTA, shared memory bytes per CTA. */
  int kernel_layout;
  int kernel_u_on_chip;
  int kernel_threads;
  int kernel_smem_bytes;
} sq_info;

/* One pseudopotential type in memory, in the units the reference holds after
 * Read_Pseudopotential (PSD_OBJ, src/ilsdft.h:63-80; src/lsdft_readfiles.cc:858-1101): a radial
 * grid whose first point is r = 0, V_l in Ha (the file's r V_l in Ry divided by 2r), U_l the
 * file's u_l / r, the valence density already divided by 4 pi r^2, every array [n_r]. */
typedef struct sq_psd_desc {
  int n_r;                  /* radial points, r[0] = 0 (PSD_OBJ.size) */
  const double *r;          /* RadialGrid */
  int lmax;                 /* highest l with a potential (PSD_OBJ.lmax, 0..3) */
  int lloc;                 /* PSEUDOPOTENTIAL_LOCAL: the l whose V_l is the local part */
  int valence;              /* valence electrons per atom (.ion) */
  const double *V[4];       /* V_l, l <= lmax (PSD_OBJ.V) */
  const double *U[4];       /* U_l, l <= lmax and l != lloc (PSD_OBJ.U); NULL otherwise */
  double rc[4];             /* cutoff radius of U_l (PSD_OBJ.rc) */
  const double *rho_atom;   /* isolated-atom valence density (PSD_OBJ.uu); NULL = zero */
} sq_psd_desc;

/* A whole cell in memory: the fields of the reference's LSDFT_OBJ (src/ilsdft.h:85-458) that
 * its input readers fill (src/lsdft_readfiles.cc:21-789), with the same meanings as the deck
 * keywords.  Zero SCF fields take the reference's defaults (readfiles.cc:62-102). */
typedef struct sq_system_desc {
  int fd_order;             /* FD_ORDER (even, 12 for the reference's stencil) */
  int bc;                   /* BOUNDARY_CONDITION 1..4 */
  double cell_half[3];      /* CELL: half side lengths R (bohr) */
  int grid[3];              /* FD_GRID */
  double beta;              /* BETA (1/Ha) */
  double rcut;              /* RADIUS_TRUNC (bohr) */
  int n_qp;                 /* LANCZOS_DEGREE, 1..64 */
  int n_types;              /* NTYPE, 1..8 */
  const sq_psd_desc *psd;   /* [n_types] */
  int n_atoms;
  const int *atom_type;     /* [n_atoms], 0..n_types-1 */
  const double *atom_xyz;   /* [n_atoms][3], centred coordinates in [-R, R) (bohr) */
  double mixing_parameter;  /* MIXING_PARAMETER (0: 0.3) */
  int mixing_history;       /* MIXING_HISTORY (0: 7) */
  int pulay_frequency;      /* PULAY_FREQUENCY (0: 1) */
  double tol_scf;           /* TOL_SCF (0: 1e-6) */
  int maxit_scf;            /* MAXIT_SCF (0: 100) */
  double reference_cutoff;  /* REFERENCE_CUTOFF (0: 0.5) */
} sq_system_desc;

/* Build the engine from a cell in memory: the same engine sq_create_from_deck builds from the
 * deck files holding these values.  Every array is copied; the caller may free them after the
 * call.  Replaces Initialize's readers for a caller that already holds an initialized
 * LSDFT_OBJ (src/main.cc:21-33, src/lsdft_initObjs.cc:36-93). */
sq_status sq_create(const sq_system_desc *sys, const sq_options *opt, sq_handle **out);
/* Host-only setup report of an in-memory cell, as sq_describe_deck for a deck. */
sq_status sq_describe_system(const sq_system_desc *sys, int faithful, sq_info *info,
                             double *gamma, double *cutoff);

/* Read <deck_dir>/<name>.inpt/.ion/.relax and <deck_dir>/pseudopotential/<psd> and build the
 * engine.  Replaces Get_Input + Initialize + GetInfluencingAtoms_Nonlocal +
 * CalculateNonlocalProjectors + NonlocalProjectors (src/main.cc:32-44,
 * src/lsdft_initObjs.cc:36-93,1671-1946, src/lsdft_nl.cc:6-208). */
sq_status sq_create_from_deck(const char *deck_dir, const char *name, const sq_options *opt,
                              sq_handle **out);
void sq_destroy(sq_handle *h);

/* Host-only setup report (no GPU touched): parse the deck and run the host setup, then fill
 * info (precision/device fields 0), gamma[n_types*4] (Gamma_l, 0 for the local l;
 * src/lsdft_initObjs.cc:822-869) and cutoff[n_types*3] (pseudocharge cutoff per axis;
 * src/lsdft_initObjs.cc:628-817).  gamma and cutoff may be NULL. */
sq_status sq_describe_deck(const char *deck_dir, const char *name, int faithful, sq_info *info,
                           double *gamma, double *cutoff);
sq_status sq_get_info(const sq_handle *h, sq_info *info);

/* Host-only plan (no GPU touched): the info an engine built from this deck with these options
 * would report on a device of num_sms SMs, smem_optin bytes of opt-in shared memory per block
 * and l2_bytes of L2, including the kernel_* fields (on-chip layout, projector-list format,
 * threads, shared memory).  A cell that fits no layout fails as sq_create_from_deck would. */
sq_status sq_plan_kernel(const char *deck_dir, const char *name, const sq_options *opt,
                         int num_sms, int smem_optin, int l2_bytes, sq_info *info);

/* Per-node Lanczos + Gauss quadrature for nodes [node_begin, node_end) in the reference's
 * node order (z slowest, x fastest; src/lsdft_scf.cc:60-67).  Replaces
 * NodesAndWeights_LSSGQ (src/lsdft.h:132, called at src/main.cc:54), which loops
 * CalculateSpectralNodesAndWeights (src/lsdft.h:131) with Mult_NonlocalVector
 * (src/lsdft.h:25) and TridiagEigenVecSolve_NodesAndWeights (src/lsdft.h:163-164).
 * HOST buffers: veff[grid] (NULL = the constant veff_const on every cube point, the
 * reference's placeholder is 0.333, src/lsdft_scf.cc:71), lambda/weights
 * [node_end-node_begin][n_qp], lambda_min/lambda_max [node_end-node_begin].
 * Host<->device copies happen inside the call. */
sq_status sq_nodes_and_weights(sq_handle *h, const double *veff, double veff_const,
                               long node_begin, long node_end, double *lambda, double *weights,
                               double *lambda_min, double *lambda_max);

/* The same on DEVICE buffers, asynchronous on `stream` (a cudaStream_t, NULL = the legacy
 * default stream).  d_veff may be NULL (constant veff_const). */
sq_status sq_nodes_and_weights_device(sq_handle *h, const double *d_veff, double veff_const,
                                      long node_begin, long node_end, double *d_lambda,
                                      double *d_weights, double *d_lambda_min,
                                      double *d_lambda_max, void *stream);

/* Wait for `stream` and report the device-side status of the preceding device calls
 * (capacity overflow, Lanczos breakdown, QL non-convergence, device timeout). */
sq_status sq_sync_status(sq_handle *h, void *stream);

/* Gauss quadrature of given tridiagonals: implicit QL on a[i][0..n_qp) (diagonal) and
 * b[i][0..n_qp-1) (sub-diagonal; b[i][n_qp-1] is ignored, as the reference zeroes it), giving
 * lambda, weights [n_nodes][n_qp] and lambda_min / lambda_max [n_nodes].  HOST buffers; runs
 * on `device`.  Replaces TridiagEigenVecSolve_NodesAndWeights (src/lsdft.h:163-164,
 * src/lsdft_tools.cc:912-1026), which exit(1)s after 50 sweeps (:950-952); here every node's
 * outputs are written and SQ_NO_CONVERGENCE is returned if any node needed more. */
sq_status sq_tridiag_nodes_and_weights(const double *a, const double *b, long n_nodes, int n_qp,
                                       double *lambda, double *weights, double *lambda_min,
                                       double *lambda_max, int device);

/* Copy the Lanczos coefficients a_k, b_k (k < n_qp) of the last nodes_and_weights call to
 * host arrays [n][n_qp] (the lssgq recurrence of src/lsdft_scf.cc:111-150). */
sq_status sq_copy_lanczos_coefficients(sq_handle *h, double *a, double *b, long n);

/* Fermi level by bisection, node densities and band energy (FP64), from the quadrature of
 * the nodes: N_e(lf) = 2 sum_nodes sum_q w f(lambda - lf), rho = (2/dV) sum_q w f,
 * e_band = 2 sum w lambda f, ts = (2/beta) sum w [f ln f + (1-f) ln(1-f)].
 * Implements the API that src/lsdft.h:98-102,209 declares (constraint_lssgq, FermiDirac,
 * CalculateDensity_lssgq, findRootBrent, SystemEnergy_Calc_lssgq) but never defines.
 * HOST buffers: lambda, weights [n_nodes][n_qp]; rho [n_nodes] (may be NULL). */
sq_status sq_fermi_density_energy(sq_handle *h, const double *lambda, const double *weights,
                                  long n_nodes, double n_electrons, double tol,
                                  double *lambda_f, double *rho, double *e_band, double *ts);

/* The same on DEVICE buffers (d_rho may be NULL); scalars are returned to host memory.
 * Synchronises `stream` before returning. */
sq_status sq_fermi_density_energy_device(sq_handle *h, const double *d_lambda,
                                         const double *d_weights, long n_nodes,
                                         double n_electrons, double tol, double *lambda_f,
                                         double *d_rho, double *e_band, double *ts,
                                         void *stream);

/* Electron count N_e(lambda_f) = 2 sum_nodes sum_q w f(lambda - lambda_f) over DEVICE buffers
 * [n_nodes][n_qp], returned to host memory: the constraint function the reference declares as
 * constraint_lssgq (src/lsdft.h:98).  One scalar per call: the local term of a Fermi
 * bisection whose nodes are sharded over several GPUs (sum over ranks, then bisect).
 * Synchronises `stream`. */
sq_status sq_electron_count_device(sq_handle *h, const double *d_lambda, const double *d_weights,
                                   long n_nodes, double lambda_f, double *count, void *stream);

/* Mixed-cell batch: every node of n_cells independent cells (each its own handle, with its
 * own mesh, Rcut, N_qp and precision) in one submission.  The reference runs one cell per job
 * (NodesAndWeights_LSSGQ, src/lsdft.h:132).  The GPU's SMs are split between the cells so that
 * they finish together: by each cell's measured cost per node and SM once every handle has run
 * before, else by its algorithmic FLOPs per node (at least one SM each).  Each cell's
 * persistent Lanczos kernel runs on its handle's stream on its share of SMs, concurrently with
 * the others, and `stream` waits for all of them.  Per cell c: d_veff[c] (DEVICE, NULL =
 * constant veff_const[c]; d_veff and veff_const may be NULL), outputs d_lambda[c],
 * d_weights[c] [n_nodes][n_qp], d_lambda_min[c], d_lambda_max[c] [n_nodes].  Synchronises the
 * cells' streams to report their status. */
sq_status sq_batch_nodes_and_weights(sq_handle *const *cells, int n_cells,
                                     const double *const *d_veff, const double *veff_const,
                                     double *const *d_lambda, double *const *d_weights,
                                     double *const *d_lambda_min, double *const *d_lambda_max,
                                     void *stream);

/* Device time (ms) of the kernels of the last nodes_and_weights call, measured with CUDA
 * events on the stream they ran on: ms[0] Lanczos kernel, ms[1] quadrature kernel. */
sq_status sq_last_kernel_times(sq_handle *h, double *ms);

/* Fault-injection self-test of the bounded device-side waits (no counterpart in the reference,
 * which has no device code): runs the Fermi-level kernel on a small synthetic input with one
 * CTA leaving before the first grid barrier and a short poll limit.  The other CTAs give up
 * after about 0.4 ms of polling and return, so the call returns SQ_DEVICE_TIMEOUT and the
 * context stays usable; SQ_OK would mean the wait did not report its timeout. */
sq_status sq_fermi_timeout_selftest(int device);

/* Measure the FP32 FMA throughput of the device (TFLOP/s) with a register-resident FMA
 * chain on every SM; the peak against which the FP32 Lanczos kernel is reported. */
sq_status sq_measure_fp32_peak(int device, double *tflops);

/* Allocation-free form of sq_fermi_density_energy_device; no counterpart in the reference.
 * For callers that must not allocate device memory (a host framework that owns the device
 * allocator, a fixed memory budget, or a stream-ordered pipeline that cannot afford the
 * allocator's implicit synchronisation): no handle, no cudaMalloc/cudaFree; the kernel runs
 * on a static scratch array of the library (about 410 KiB per GPU, held until exit).
 * DEVICE inputs d_lambda, d_weights [n_nodes][n_qp]; d_rho [n_nodes] may be NULL; the
 * HOST array out[3] receives lambda_f, e_band and ts; maxit <= 200 (else SQ_CAPACITY).
 * Every call looks the array's address up in the current context (no allocation).  Calls
 * share the array: calls that overlap on the GPU race.  Synchronises `stream` before
 * returning, so it cannot be called while `stream` is being captured (SQ_BAD_INPUT).
 * SQ_NO_CONVERGENCE (out[] still filled with the last midpoint) when the bisection used all
 * maxit steps without narrowing the bracket below tol. */
sq_status sq_fermi_density_energy_noalloc(const double *d_lambda, const double *d_weights,
                                          long n_nodes, int n_qp, double beta,
                                          double n_electrons, double dV, double tol, int maxit,
                                          double *d_rho, double *out, void *stream);

/* ---- SCF closure (periodic decks, BOUNDARY_CONDITION 2) ----
 * The self-consistent loop that the reference declares as SCF_LSSGQ (src/lsdft.h:153) with
 * SolvePoisson (:93), mix (:183), Vxc_Calc_CA_PW / Exc_Calc_CA_PW (:201-202) and
 * SystemEnergy_Calc_lssgq (:209), none of which has a body in the reference.  One iteration:
 * pseudocharge Poisson solve of the FD Laplacian (exact, in Fourier space), LDA
 * (Slater + Perdew-Wang 92) potential, the per-node Lanczos/quadrature pass with that Veff,
 * Fermi bisection, density residual, Harris-Foulkes free energy and Periodic-Pulay mixing
 * (MIXING_PARAMETER / MIXING_HISTORY / PULAY_FREQUENCY, src/lsdft_readfiles.cc:219-228). */
typedef struct sq_scf_options {
  double tol;               /* ||rho_out - rho_in|| / ||rho_out|| target; <= 0: TOL_SCF;
                               raised to 3e-5 for an FP32 engine */
  int maxit;                /* <= 0: MAXIT_SCF */
  double mixing_parameter;  /* <= 0: MIXING_PARAMETER */
  int mixing_history;       /* <= 0: MIXING_HISTORY (at most 16) */
  int pulay_frequency;      /* <= 0: PULAY_FREQUENCY */
  double fermi_tol;         /* bisection tolerance on lambda_f; <= 0: 1e-12 */
  double kerker_ktf;        /* Kerker preconditioner k_TF (1/bohr) of the mixing: > 0 that value,
                               0 the default 1.0 (the reference mixes preconditioned,
                               src/lsdft_readfiles.cc:102), < 0 no preconditioner */
  int cuda_graph;           /* 1: from the second iteration on, replay one captured CUDA graph
                               of the iteration's device part (Poisson, potential, Lanczos,
                               quadrature); 0: direct launches */
  double learned_highpass;  /* sq_scf_begin_learned only: > 0 keeps of the network's correction
                               to the atomic superposition only its short wavelengths, scaled
                               by k^2 / (k^2 + k0^2) with k0 this value (1/bohr); 0 the whole
                               correction */
} sq_scf_options;

typedef struct sq_scf_result {
  int iterations;          /* SCF iterations done since sq_scf_begin */
  int converged;           /* 1 once the residual is below tol */
  double free_energy;      /* Ha: e_band + e_xc - e_xc_dc + e_electrostatic - e_self + e_corr + ts */
  double free_energy_per_atom;
  double e_band;           /* 2 sum w lambda f */
  double e_xc;             /* int rho_in eps_xc(rho_in) */
  double e_xc_dc;          /* int rho_in Vxc(rho_in) */
  double e_electrostatic;  /* 1/2 int (b - rho_in) phi */
  double e_self;           /* 1/2 sum_J int b_J V_J */
  double e_corr;           /* overlap correction of the pseudocharges */
  double ts;               /* -TS = (2/beta) sum w [f ln f + (1-f) ln(1-f)] */
  double lambda_f;         /* Fermi level */
  double residual;         /* ||rho_out - rho_in|| / ||rho_out|| of the last iteration */
  double seconds;          /* host wall time of the iterations since sq_scf_begin */
  double sq_ms;            /* device time of the Lanczos + quadrature kernels, summed */
  double tol;              /* residual target in force: the requested one, but at least 3e-5
                              with FP32 Lanczos vectors (their residual noise floor is ~1e-5) */
} sq_scf_result;

/* ---- One SCF iteration with the FD nodes sharded over ranks, one GPU per rank ----
 * The reference splits the nodes of one cell over MPI ranks (DMDACreate3d on
 * PETSC_COMM_WORLD, src/lsdft_initObjs.cc:132-133; each rank loops over its corner block,
 * src/lsdft_scf.cc:47-62).  Here every rank holds the whole cell (handle + sq_scf_begin with
 * the same options and start density, so the replicated fields stay identical), runs the SQ
 * pass on its node range only, and the caller supplies the three exchanges with its own
 * collectives (the Python driver sqminiapp_gb300.sharding.ShardedSCF uses torch.distributed):
 *   1. sq_scf_shard_sq: potential of rho_in (replicated), then Lanczos + quadrature of nodes
 *      [node_begin, node_end); minmax[2] = this range's smallest and largest Ritz value;
 *   2. the Fermi level from sq_scf_shard_counts (this range's electron counts at k trial
 *      levels, summed over ranks by the caller), as many rounds as the search needs;
 *   3. sq_scf_shard_density: this range's node densities (HOST rho_local[node_end-node_begin])
 *      and sums[2] = its partial band energy 2 sum w lambda f and entropy sum
 *      2 sum w [f ln f + (1-f) ln(1-f)] (summed over ranks; -TS is the second sum / beta);
 *   4. sq_scf_shard_finish with the gathered full HOST rho_out[n_nodes] and the summed
 *      scalars: residual, free energy and Periodic-Pulay mixing, replicated on every rank.
 * No call waits on another rank. */
sq_status sq_scf_shard_sq(sq_handle *h, long node_begin, long node_end, double *minmax);
sq_status sq_scf_shard_counts(sq_handle *h, int k, const double *lambda_f, double *counts);
sq_status sq_scf_shard_density(sq_handle *h, double lambda_f, double *rho_local, double *sums);
sq_status sq_scf_shard_finish(sq_handle *h, const double *rho_out, double lambda_f, double e_band,
                              double ts, sq_scf_result *result);

/* Host-only report of a periodic deck's fixed SCF fields (no GPU touched): pseudocharges
 * b[n_nodes], atomic-superposition density rho0[n_nodes], the Poisson symbol green on the
 * R2C half grid [Nz][Ny][Nx/2+1], and scalars[4] = E_self, E_self of the reference
 * pseudocharges, E_c, int b.  Any output may be NULL. */
sq_status sq_describe_scf_fields(const char *deck_dir, const char *name, double *b, double *rho0,
                                 double *green, double *scalars);
/* Start an SCF: rho_init HOST [n_nodes] (NULL = superposition of the psd atomic valence
 * densities, SuperposAtRho of src/ilsdft.h:269), cut at zero and scaled to the electron
 * count.  opt may be NULL (deck values).  Clears the mixing history. */
sq_status sq_scf_begin(sq_handle *h, const sq_scf_options *opt, const double *rho_init);
/* The same with a DEVICE initial density (a learned or checkpointed guess). */
sq_status sq_scf_begin_device(sq_handle *h, const sq_scf_options *opt, const double *d_rho_init);
/* One SCF iteration; result (may be NULL) receives the state after it. */
sq_status sq_scf_step(sq_handle *h, sq_scf_result *result);
/* sq_scf_begin, then iterate until converged (SQ_OK) or MAXIT_SCF (SQ_NO_CONVERGENCE). */
sq_status sq_scf_run(sq_handle *h, const sq_scf_options *opt, const double *rho_init,
                     sq_scf_result *result);
/* HOST copies [n_nodes] of the last output density and of the next input density (either
 * may be NULL). */
sq_status sq_scf_get_density(sq_handle *h, double *rho_out, double *rho_in);
/* HOST copies [n_nodes] of the pseudocharge b, the initial density, and the phi / Vxc of the
 * last iteration (any may be NULL); scalars[4] = E_self, E_self of the reference
 * pseudocharges, E_c, int b. */
sq_status sq_scf_get_fields(sq_handle *h, double *b, double *rho0, double *phi, double *vxc,
                            double *scalars);
/* Free energy and residual of every iteration since sq_scf_begin (up to cap entries). */
sq_status sq_scf_history(sq_handle *h, int cap, double *free_energy, double *residual, int *count);
/* Host evaluation of the LDA functional the SCF uses: eps_xc and Vxc per density value. */
sq_status sq_lda_pw92(const double *rho, long n, double *eps, double *v);

/* ---- Learned warm start (no counterpart in the reference, whose SCF starts from the atomic
 * superposition, SuperposAtRho, src/ilsdft.h:269).  A 64-128-128-1 MLP with SiLU activations
 * maps 64 rotation-invariant neighbour descriptors of each grid point (16 Gaussian radial
 * centres over 0-8 bohr times l = 0..3) to the correction rho_SCF - rho_0; BF16 weights and
 * activations, FP32 accumulation on the tensor cores (tcgen05), Adam training on the GPU. */
typedef struct sq_mlp sq_mlp;
#define SQ_MLP_N_PARAMS 24961  /* W1[64][128], b1[128], W2[128][128], b2[128], w3[128], b3 */
/* A network with He-initialised weights on `device`. */
sq_status sq_mlp_create(int device, unsigned long long seed, sq_mlp **out);
void sq_mlp_destroy(sq_mlp *m);
sq_status sq_mlp_save(const sq_mlp *m, const char *path);
sq_status sq_mlp_load(const char *path, int device, sq_mlp **out);
/* FP32 master parameters (SQ_MLP_N_PARAMS, layout above), feature standardisation
 * (mean[64], 1/std[64]; NULL keeps the current one) and target scale. */
sq_status sq_mlp_set_params(sq_mlp *m, const float *params, const float *feat_mean,
                            const float *feat_inv_std, double t_mean, double t_std);
sq_status sq_mlp_get_params(const sq_mlp *m, float *params, float *feat_mean,
                            float *feat_inv_std, double *t_mean, double *t_std);
/* Raw descriptors of every node of the handle's cell, HOST [n_nodes][64]. */
sq_status sq_descriptors(sq_handle *h, float *desc);
/* Add the handle's cell as training samples: descriptors and rho_out - rho_0 of its last SCF. */
sq_status sq_mlp_add_training_cell(sq_mlp *m, sq_handle *h);
/* Adam steps (tiles_per_step tiles of 128 samples each step, learning rate lr); the first
 * call fixes the standardisation from the samples.  final_loss: mean squared error of the
 * last step in standardised units. */
sq_status sq_mlp_train(sq_mlp *m, int steps, int tiles_per_step, double lr, double *final_loss);
/* Loss and gradients (SQ_MLP_N_PARAMS) of mean((y - t)^2) over n standardised samples
 * x [n][64], t [n] (HOST), computed by the tensor-core training kernel. */
sq_status sq_mlp_gradients(sq_mlp *m, const float *x, const float *t, long n, double *loss,
                           float *grads);
/* Network outputs y [n] (standardised units) of standardised features x [n][64] (HOST). */
sq_status sq_mlp_forward(sq_mlp *m, const float *x, long n, float *y);
/* Predicted density rho_0 + correction of the handle's cell, HOST [n_nodes]. */
sq_status sq_mlp_predict_density(sq_mlp *m, sq_handle *h, double *rho);
/* sq_scf_begin from the network's predicted density (cut at zero, scaled to N_e). */
sq_status sq_scf_begin_learned(sq_handle *h, const sq_scf_options *opt, sq_mlp *m);

/* ---- The reference's text files (one block of the grid per rank; one GPU: corner 0, dims =
 * FD_GRID).  Files are "<prefix>_<rank>.den" / ".lambdas"; reading fails with SQ_BAD_INPUT
 * when the header's block differs from corner/dims. */
/* Print_ElecDens (src/lsdft_readfiles.cc:1106-1138): header "xcor ycor zcor lx ly lz", then
 * "k j i value" (%0.16lf) per point; rho is HOST [dims[2]][dims[1]][dims[0]]. */
sq_status sq_write_density_file(const char *prefix, int rank, const int corner[3],
                                const int dims[3], const double *rho);
/* Read_ElecDens (:1242-1289): the inverse; a density to restart an SCF from. */
sq_status sq_read_density_file(const char *prefix, int rank, const int corner[3],
                               const int dims[3], double *rho);
/* Print_MinMaxLambda / Read_MinMaxLambda (:1294-1381): "LIpos lambda_min lambda_max". */
sq_status sq_write_lambda_file(const char *prefix, int rank, const int corner[3],
                               const int dims[3], const double *lambda_min,
                               const double *lambda_max);
sq_status sq_read_lambda_file(const char *prefix, int rank, const int corner[3],
                              const int dims[3], double *lambda_min, double *lambda_max);
/* The input-parameter and initialization echo of the reference's .out file
 * (src/lsdft_readfiles.cc:520-607) for the keywords this engine reads. */
sq_status sq_write_output_echo(const sq_handle *h, const char *path);

/* Message of the last failing call on this thread. */
const char *sq_last_error_string(void);

#ifdef __cplusplus
}
#endif
#endif
