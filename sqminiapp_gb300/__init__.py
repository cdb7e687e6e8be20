"""GB300 Spectral Quadrature engine: Python mirror of the reference's per-node SQ API.

The compute path is the in-tree CUDA library ``lib/libsq_gb300.so`` (sm_103a) behind the
C ABI of ``include/sq_gb300.h``; this module only binds it with ctypes.  There is no CPU
fallback: if the library is missing the import of :class:`LSDFT` fails loudly.

Names follow the reference (SQMiniApp ``src/lsdft.h``):

* ``LSDFT(deck_dir, name)``         -- Get_Input + Initialize + GetInfluencingAtoms_Nonlocal +
                                       CalculateNonlocalProjectors + NonlocalProjectors
                                       (src/main.cc:32-44)
* ``LSDFT.NodesAndWeights_LSSGQ``   -- src/lsdft_scf.cc:32-82 (per-node Lanczos + quadrature)
* ``LSDFT.CalculateDensity_lssgq``  -- declared at src/lsdft.h:100 (Fermi bisection, density,
                                       band energy), implemented from the SQ method
* ``LSDFT.SCF_LSSGQ``               -- declared at src/lsdft.h:153 (the SCF loop: Poisson,
                                       LDA, SQ pass, Fermi level, energy, Periodic Pulay)
"""
import ctypes
import os

import numpy as np

from .capi import SQ_OK, SqError, SqInfo, SqOptions, SqScfOptions, SqScfResult, lib, check, library_path

__all__ = ["LSDFT", "SqError", "library_path", "DECK_DIR", "lda_pw92", "Print_ElecDens",
           "Read_ElecDens", "Print_MinMaxLambda", "Read_MinMaxLambda", "WarmStartMLP",
           "batch_nodes_and_weights", "plan_kernel", "GB300_DEVICE"]

# SM count, opt-in shared memory per block and L2 size of a GB300, for plan_kernel.
GB300_DEVICE = {"num_sms": 152, "smem_optin": 232448, "l2_bytes": 126 * 1024 * 1024}

DECK_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "decks")

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _fptr(a):
    return a.ctypes.data_as(_fp)


class LSDFT:
    """One SQ engine on one GPU, built from a reference input deck.

    faithful=True keeps the reference operator with its quirks (shared projector
    coefficient per atom, pseudocharge-based image range); faithful=False (default) is the
    corrected operator.  precision=32 runs FP32 Lanczos vectors with FP64 recurrence
    coefficients, quadrature and sums; precision=64 is FP64 throughout.  list_format picks
    the FP32 corrected operator's projector-list records (0 automatic, 1 full chi_lm, 2
    compact radial values; sq_options.list_format); kernel the FP32 Lanczos kernel (0
    automatic, 1 single-pass, 2 split-pass) and tile the split-pass kernel's z-/y-ranges per
    row (0: timed on the first call).
    """

    def __init__(self, deck_dir, name, faithful=False, precision=32, device=0, list_format=0,
                 kernel=0, tile=0, system=None):
        """deck_dir/name: the reference's input deck; or deck_dir=name=None and system=a cell
        in memory (sqminiapp_gb300.system.read_system's dict), built with sq_create."""
        self._lib = lib()
        self._h = ctypes.c_void_p()
        opt = SqOptions(int(bool(faithful)), int(precision), int(device), int(list_format),
                        int(kernel), int(tile))
        if system is not None:
            from .system import to_desc
            packed = to_desc(system)
            check(self._lib.sq_create(ctypes.byref(packed.desc), ctypes.byref(opt),
                                      ctypes.byref(self._h)), "sq_create")
        else:
            check(self._lib.sq_create_from_deck(deck_dir.encode(), name.encode(),
                                                ctypes.byref(opt), ctypes.byref(self._h)),
                  "sq_create_from_deck")
        info = SqInfo()
        check(self._lib.sq_get_info(self._h, ctypes.byref(info)), "sq_get_info")
        self.info = info
        self.grid = tuple(info.grid)
        self.cube = tuple(info.cube)
        self.n_qp = info.n_qp
        self.n_nodes = info.n_nodes
        self.h = tuple(info.h)
        self.dV = info.dV
        self.beta = info.beta
        self.n_electrons = info.n_electrons
        self.precision = precision
        self.faithful = bool(faithful)

    def close(self):
        if self._h:
            self._lib.sq_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- per-node Lanczos + Gauss quadrature -------------------------------------------
    def NodesAndWeights_LSSGQ(self, veff=None, veff_const=0.333, node_begin=0, node_end=None,
                              out=None):
        """Quadrature nodes/weights of nodes [node_begin, node_end) (host arrays).

        veff: None for a constant ``veff_const`` (the reference's placeholder is 0.333,
        src/lsdft_scf.cc:71) or an array over the FD grid (z slowest, x fastest).
        out: optional dict of preallocated float64 arrays (e.g. pinned memory) with keys
        lambda, weights [n, n_qp] and lambda_min, lambda_max [n]."""
        if node_end is None:
            node_end = self.n_nodes
        n = node_end - node_begin
        if out is None:
            lam = np.empty((n, self.n_qp))
            w = np.empty((n, self.n_qp))
            lmin = np.empty(n)
            lmax = np.empty(n)
        else:
            lam, w, lmin, lmax = out["lambda"], out["weights"], out["lambda_min"], out["lambda_max"]
            for a, shape in ((lam, (n, self.n_qp)), (w, (n, self.n_qp)), (lmin, (n,)), (lmax, (n,))):
                if a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError("out arrays must be C-contiguous float64 of the right shape")
        vp = None
        if veff is not None:
            veff = np.ascontiguousarray(veff, dtype=np.float64).reshape(-1)
            if veff.size != self.n_nodes:
                raise ValueError("veff must have one value per FD node")
            vp = _ptr(veff)
        check(self._lib.sq_nodes_and_weights(self._h, vp, float(veff_const), int(node_begin),
                                             int(node_end), _ptr(lam), _ptr(w), _ptr(lmin),
                                             _ptr(lmax)), "sq_nodes_and_weights")
        return {"lambda": lam, "weights": w, "lambda_min": lmin, "lambda_max": lmax}

    def nodes_and_weights_device(self, d_veff, veff_const, node_begin, node_end, d_lambda,
                                 d_weights, d_lmin, d_lmax, stream=0):
        """Asynchronous device-pointer form (integers are raw CUDA device addresses)."""
        check(self._lib.sq_nodes_and_weights_device(
            self._h, ctypes.c_void_p(d_veff) if d_veff else None, float(veff_const),
            int(node_begin), int(node_end), ctypes.c_void_p(d_lambda), ctypes.c_void_p(d_weights),
            ctypes.c_void_p(d_lmin), ctypes.c_void_p(d_lmax), ctypes.c_void_p(stream)),
            "sq_nodes_and_weights_device")

    def last_kernel_times(self):
        """(lanczos_ms, quadrature_ms) of the last nodes-and-weights call (CUDA events)."""
        ms = np.zeros(2)
        check(self._lib.sq_last_kernel_times(self._h, _ptr(ms)), "sq_last_kernel_times")
        return float(ms[0]), float(ms[1])

    def algorithmic_flops_per_node(self):
        """Useful FP32 FLOPs of one node's Lanczos (n_qp matvecs): per step 2(6o+1) per cube
        point for the stencil, 1 for Veff, 8 for the recurrence's vector updates and
        products, and 4 per projector-point-(l,m) for the nonlocal gather and scatter."""
        nc = self.cube[0] * self.cube[1] * self.cube[2]
        o = self.info.fd_half_order
        per_step = (2 * (6 * o + 1) + 1 + 8) * nc + 4 * self.info.n_lm * self.info.proj_points_per_node
        return self.n_qp * per_step

    def sync_status(self, stream=0):
        check(self._lib.sq_sync_status(self._h, ctypes.c_void_p(stream)), "sq_sync_status")

    def lanczos_coefficients(self, n):
        """a_k, b_k (k < n_qp) of the first n nodes of the last call."""
        a = np.empty((n, self.n_qp))
        b = np.empty((n, self.n_qp))
        check(self._lib.sq_copy_lanczos_coefficients(self._h, _ptr(a), _ptr(b), int(n)),
              "sq_copy_lanczos_coefficients")
        return a, b

    # --- Fermi level, density, energy ----------------------------------------------------
    def CalculateDensity_lssgq(self, lam, weights, n_electrons=None, tol=1e-12, rho=None):
        """Fermi level by bisection, node densities, band energy and -TS (FP64)."""
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        n_nodes = lam.shape[0]
        if n_electrons is None:
            n_electrons = self.n_electrons
        if rho is None:
            rho = np.empty(n_nodes)
        lf = ctypes.c_double()
        eb = ctypes.c_double()
        ts = ctypes.c_double()
        check(self._lib.sq_fermi_density_energy(self._h, _ptr(lam), _ptr(weights), n_nodes,
                                                float(n_electrons), float(tol), ctypes.byref(lf),
                                                _ptr(rho), ctypes.byref(eb), ctypes.byref(ts)),
              "sq_fermi_density_energy")
        return {"lambda_f": lf.value, "rho": rho, "e_band": eb.value, "ts": ts.value}

    def electron_count_device(self, d_lambda, d_weights, n_nodes, lambda_f, stream=0):
        """N_e(lambda_f) of device quadrature arrays (constraint_lssgq, src/lsdft.h:98)."""
        c = ctypes.c_double()
        check(self._lib.sq_electron_count_device(self._h, ctypes.c_void_p(d_lambda),
                                                 ctypes.c_void_p(d_weights), int(n_nodes),
                                                 float(lambda_f), ctypes.byref(c),
                                                 ctypes.c_void_p(stream)),
              "sq_electron_count_device")
        return c.value

    def fermi_density_energy_device(self, d_lambda, d_weights, n_nodes, n_electrons, tol,
                                    d_rho, stream=0):
        lf = ctypes.c_double()
        eb = ctypes.c_double()
        ts = ctypes.c_double()
        check(self._lib.sq_fermi_density_energy_device(
            self._h, ctypes.c_void_p(d_lambda), ctypes.c_void_p(d_weights), int(n_nodes),
            float(n_electrons), float(tol), ctypes.byref(lf),
            ctypes.c_void_p(d_rho) if d_rho else None, ctypes.byref(eb), ctypes.byref(ts),
            ctypes.c_void_p(stream)), "sq_fermi_density_energy_device")
        return {"lambda_f": lf.value, "e_band": eb.value, "ts": ts.value}

    # --- SCF closure (SCF_LSSGQ, src/lsdft.h:153) -----------------------------------------
    @staticmethod
    def _scf_options(tol, maxit, mixing_parameter, mixing_history, pulay_frequency, fermi_tol,
                     kerker_ktf=None, cuda_graph=False, learned_highpass=None):
        return SqScfOptions(float(tol or 0.0), int(maxit or 0), float(mixing_parameter or 0.0),
                            int(mixing_history or 0), int(pulay_frequency or 0),
                            float(fermi_tol or 0.0), float(kerker_ktf or 0.0),
                            int(bool(cuda_graph)), float(learned_highpass or 0.0))

    def SCF_LSSGQ(self, rho_init=None, tol=None, maxit=None, mixing_parameter=None,
                  mixing_history=None, pulay_frequency=None, fermi_tol=None, kerker_ktf=None,
                  raise_on_maxit=True, model=None, cuda_graph=False, learned_highpass=None):
        """Self-consistent field loop on the GPU until ||rho_out - rho_in|| / ||rho_out|| < tol.

        rho_init: None (superposition of atomic valence densities) or a host density over the
        FD grid.  None for any option takes the deck's value (TOL_SCF, MAXIT_SCF,
        MIXING_PARAMETER, MIXING_HISTORY, PULAY_FREQUENCY); kerker_ktf None/0 = Kerker with
        k_TF = 1/bohr, negative = unpreconditioned mixing.  Returns the result dict of the
        last iteration with the per-iteration history of free energy and residual."""
        opt = self._scf_options(tol, maxit, mixing_parameter, mixing_history, pulay_frequency,
                                fermi_tol, kerker_ktf, cuda_graph, learned_highpass)
        if model is not None:
            # learned start (sq_scf_begin_learned), then the same loop one step at a time
            check(self._lib.sq_scf_begin_learned(self._h, ctypes.byref(opt), model._m),
                  "sq_scf_begin_learned")
            limit = self._deck_maxit() if not maxit else int(maxit)
            out = {}
            for _ in range(limit):
                out = self.scf_step()
                if out["converged"]:
                    break
            if not out.get("converged") and raise_on_maxit:
                raise SqError(2, "SCF_LSSGQ", "SCF did not reach TOL_SCF within MAXIT_SCF iterations")
            out["free_energy_history"], out["residual_history"] = self.scf_history()
            return out
        rp = None
        if rho_init is not None:
            rho_init = np.ascontiguousarray(rho_init, dtype=np.float64).reshape(-1)
            if rho_init.size != self.n_nodes:
                raise ValueError("rho_init must have one value per FD node")
            rp = _ptr(rho_init)
        res = SqScfResult()
        st = self._lib.sq_scf_run(self._h, ctypes.byref(opt), rp, ctypes.byref(res))
        if st != SQ_OK and not (st == 2 and not raise_on_maxit):
            check(st, "sq_scf_run")
        out = res.as_dict()
        out["free_energy_history"], out["residual_history"] = self.scf_history()
        return out

    def _deck_maxit(self):
        # MAXIT_SCF of the deck is not in sq_info; a learned start runs at most 100 steps by
        # default, the reference's MAXIT_SCF default
        return 100

    def descriptors(self):
        """The 64 neighbour descriptors of every node [n_nodes, 64] (FP32)."""
        d = np.empty((self.n_nodes, 64), dtype=np.float32)
        check(self._lib.sq_descriptors(self._h, _fptr(d)), "sq_descriptors")
        return d

    def scf_begin(self, rho_init=None, d_rho_init=None, **opts):
        """Start an SCF by hand (then call scf_step); d_rho_init is a device address."""
        opt = self._scf_options(opts.get("tol"), opts.get("maxit"), opts.get("mixing_parameter"),
                                opts.get("mixing_history"), opts.get("pulay_frequency"),
                                opts.get("fermi_tol"), opts.get("kerker_ktf"),
                                opts.get("cuda_graph"))
        if d_rho_init is not None:
            check(self._lib.sq_scf_begin_device(self._h, ctypes.byref(opt),
                                                ctypes.c_void_p(d_rho_init)), "sq_scf_begin_device")
            return
        rp = None
        if rho_init is not None:
            rho_init = np.ascontiguousarray(rho_init, dtype=np.float64).reshape(-1)
            rp = _ptr(rho_init)
        check(self._lib.sq_scf_begin(self._h, ctypes.byref(opt), rp), "sq_scf_begin")

    def scf_step(self):
        res = SqScfResult()
        check(self._lib.sq_scf_step(self._h, ctypes.byref(res)), "sq_scf_step")
        return res.as_dict()

    def scf_history(self):
        n = ctypes.c_int()
        check(self._lib.sq_scf_history(self._h, 0, None, None, ctypes.byref(n)), "sq_scf_history")
        F = np.empty(n.value)
        E = np.empty(n.value)
        check(self._lib.sq_scf_history(self._h, n.value, _ptr(F), _ptr(E), ctypes.byref(n)),
              "sq_scf_history")
        return F, E

    def scf_density(self):
        """(rho_out of the last iteration, rho_in of the next one), host arrays."""
        ro = np.empty(self.n_nodes)
        ri = np.empty(self.n_nodes)
        check(self._lib.sq_scf_get_density(self._h, _ptr(ro), _ptr(ri)), "sq_scf_get_density")
        return ro, ri

    def write_output_echo(self, path):
        """The reference's .out header (input parameters, initialization) for this deck."""
        check(self._lib.sq_write_output_echo(self._h, str(path).encode()), "sq_write_output_echo")

    def scf_fields(self):
        """Pseudocharge b, initial density, phi and Vxc of the last iteration, and the scalars
        E_self, E_self(reference pseudocharges), E_c, int b."""
        arrs = [np.empty(self.n_nodes) for _ in range(4)]
        sc = np.empty(4)
        check(self._lib.sq_scf_get_fields(self._h, *[_ptr(a) for a in arrs], _ptr(sc)),
              "sq_scf_get_fields")
        return {"b": arrs[0], "rho0": arrs[1], "phi": arrs[2], "vxc": arrs[3],
                "e_self": sc[0], "e_self_ref": sc[1], "e_corr": sc[2], "b_total": sc[3]}


def plan_kernel(deck_dir, name, faithful=False, precision=32, list_format=0, device=None,
                kernel=0, tile=0):
    """Host-only plan (sq_plan_kernel): the SqInfo an engine for this deck would report on a
    device with the given properties (default GB300_DEVICE), kernel_* fields included."""
    dev = dict(GB300_DEVICE, **(device or {}))
    info = SqInfo()
    opt = SqOptions(int(bool(faithful)), int(precision), 0, int(list_format), int(kernel),
                    int(tile))
    check(lib().sq_plan_kernel(deck_dir.encode(), name.encode(), ctypes.byref(opt),
                               int(dev["num_sms"]), int(dev["smem_optin"]), int(dev["l2_bytes"]),
                               ctypes.byref(info)), "sq_plan_kernel")
    return info


def lda_pw92(rho):
    """The library's host evaluation of the LDA functional: (eps_xc, Vxc) per density."""
    rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
    e = np.empty_like(rho)
    v = np.empty_like(rho)
    check(lib().sq_lda_pw92(_ptr(rho), rho.size, _ptr(e), _ptr(v)), "sq_lda_pw92")
    return e, v


def _block(shape, corner):
    nz, ny, nx = shape
    c = (ctypes.c_int * 3)(*[int(v) for v in corner])
    d = (ctypes.c_int * 3)(nx, ny, nz)
    return c, d


def Print_ElecDens(prefix, rho, rank=0, corner=(0, 0, 0)):
    """Write rho [nz, ny, nx] (a rank's block) as <prefix>_<rank>.den in the reference format
    (src/lsdft_readfiles.cc:1106-1138)."""
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    c, d = _block(rho.shape, corner)
    check(lib().sq_write_density_file(str(prefix).encode(), int(rank), c, d, _ptr(rho)),
          "sq_write_density_file")


def Read_ElecDens(prefix, shape, rank=0, corner=(0, 0, 0)):
    """Read <prefix>_<rank>.den (src/lsdft_readfiles.cc:1242-1289) into [nz, ny, nx]."""
    rho = np.empty(shape)
    c, d = _block(shape, corner)
    check(lib().sq_read_density_file(str(prefix).encode(), int(rank), c, d, _ptr(rho)),
          "sq_read_density_file")
    return rho


def Print_MinMaxLambda(prefix, lambda_min, lambda_max, shape, rank=0, corner=(0, 0, 0)):
    """<prefix>_<rank>.lambdas (src/lsdft_readfiles.cc:1294-1328)."""
    lo = np.ascontiguousarray(lambda_min, dtype=np.float64).reshape(-1)
    hi = np.ascontiguousarray(lambda_max, dtype=np.float64).reshape(-1)
    c, d = _block(shape, corner)
    check(lib().sq_write_lambda_file(str(prefix).encode(), int(rank), c, d, _ptr(lo), _ptr(hi)),
          "sq_write_lambda_file")


def Read_MinMaxLambda(prefix, shape, rank=0, corner=(0, 0, 0)):
    """Read <prefix>_<rank>.lambdas (src/lsdft_readfiles.cc:1333-1381)."""
    n = int(np.prod(shape))
    lo = np.empty(n)
    hi = np.empty(n)
    c, d = _block(shape, corner)
    check(lib().sq_read_lambda_file(str(prefix).encode(), int(rank), c, d, _ptr(lo), _ptr(hi)),
          "sq_read_lambda_file")
    return lo, hi


class WarmStartMLP:
    """The learned SCF start: a 64-128-128-1 BF16 MLP trained on the GPU (tensor-core kernels)
    to predict rho_SCF - rho_0 from the 64 neighbour descriptors of each node."""

    N_PARAMS = 24961
    SHAPES = (("W1", (64, 128)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)),
              ("w3", (128,)), ("b3", (1,)))

    def __init__(self, device=0, seed=1, path=None):
        self._lib = lib()
        self._m = ctypes.c_void_p()
        if path is not None:
            check(self._lib.sq_mlp_load(str(path).encode(), int(device), ctypes.byref(self._m)),
                  "sq_mlp_load")
        else:
            check(self._lib.sq_mlp_create(int(device), int(seed), ctypes.byref(self._m)),
                  "sq_mlp_create")

    def close(self):
        if self._m:
            self._lib.sq_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self, path):
        check(self._lib.sq_mlp_save(self._m, str(path).encode()), "sq_mlp_save")

    @classmethod
    def _split(cls, flat):
        out, o = {}, 0
        for name, shape in cls.SHAPES:
            n = int(np.prod(shape))
            out[name] = flat[o:o + n].reshape(shape).copy()
            o += n
        return out

    @classmethod
    def _join(cls, params):
        return np.concatenate([np.asarray(params[n], dtype=np.float32).reshape(-1)
                               for n, _ in cls.SHAPES])

    def get_params(self):
        flat = np.empty(self.N_PARAMS, dtype=np.float32)
        mean = np.empty(64, dtype=np.float32)
        istd = np.empty(64, dtype=np.float32)
        tm, ts = ctypes.c_double(), ctypes.c_double()
        check(self._lib.sq_mlp_get_params(self._m, _fptr(flat), _fptr(mean), _fptr(istd),
                                          ctypes.byref(tm), ctypes.byref(ts)), "sq_mlp_get_params")
        p = self._split(flat)
        p.update(feat_mean=mean, feat_inv_std=istd, t_mean=tm.value, t_std=ts.value)
        return p

    def set_params(self, params, feat_mean=None, feat_inv_std=None, t_mean=0.0, t_std=1.0):
        flat = np.ascontiguousarray(self._join(params), dtype=np.float32)
        fm = None if feat_mean is None else _fptr(np.ascontiguousarray(feat_mean, np.float32))
        fi = None if feat_inv_std is None else _fptr(np.ascontiguousarray(feat_inv_std, np.float32))
        check(self._lib.sq_mlp_set_params(self._m, _fptr(flat), fm, fi, float(t_mean), float(t_std)),
              "sq_mlp_set_params")

    def gradients(self, x, t):
        """(loss, grads dict) of mean((y - t)^2) from the tensor-core training kernel."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(self.N_PARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        check(self._lib.sq_mlp_gradients(self._m, _fptr(x), _fptr(t), len(t), ctypes.byref(loss),
                                         _fptr(g)), "sq_mlp_gradients")
        return loss.value, self._split(g)

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty(len(x), dtype=np.float32)
        check(self._lib.sq_mlp_forward(self._m, _fptr(x), len(x), _fptr(y)), "sq_mlp_forward")
        return y

    def add_training_cell(self, engine):
        """Samples from an engine whose SCF has run: descriptors and rho_out - rho_0."""
        check(self._lib.sq_mlp_add_training_cell(self._m, engine._h), "sq_mlp_add_training_cell")

    def train(self, steps, tiles_per_step=152, lr=1e-3):
        loss = ctypes.c_double()
        check(self._lib.sq_mlp_train(self._m, int(steps), int(tiles_per_step), float(lr),
                                     ctypes.byref(loss)), "sq_mlp_train")
        return loss.value

    def predict_density(self, engine):
        rho = np.empty(engine.n_nodes)
        check(self._lib.sq_mlp_predict_density(self._m, engine._h, _ptr(rho)),
              "sq_mlp_predict_density")
        return rho


def batch_nodes_and_weights(engines, veffs=None, veff_consts=None, outputs=None, stream=0):
    """All nodes of several cells (one LSDFT each) in one batched submission
    (sq_batch_nodes_and_weights): the SMs are split so that the cells finish together and the
    cells' kernels run concurrently.  veffs: per cell a device address of its FD-grid Veff
    (FP64) or None; outputs: per cell a dict of device addresses lambda, weights, lambda_min,
    lambda_max.  Asynchronous on `stream` apart from the final status check."""
    n = len(engines)
    vp = ctypes.c_void_p
    hs = (vp * n)(*[e._h for e in engines])
    dv = None if veffs is None else (vp * n)(*[v or None for v in veffs])
    vc = None if veff_consts is None else (ctypes.c_double * n)(*[float(c) for c in veff_consts])
    cols = {k: (vp * n)(*[o[k] for o in outputs]) for k in ("lambda", "weights", "lambda_min",
                                                              "lambda_max")}
    check(lib().sq_batch_nodes_and_weights(hs, n, dv, vc, cols["lambda"], cols["weights"],
                                           cols["lambda_min"], cols["lambda_max"], vp(stream)),
          "sq_batch_nodes_and_weights")
