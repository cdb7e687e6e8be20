"""ctypes declarations of include/sq_gb300.h for the in-tree library lib/libsq_gb300.so."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "lib", "libsq_gb300.so")

SQ_OK = 0
SQ_BAD_INPUT = 1
SQ_NO_CONVERGENCE = 2
SQ_LANCZOS_BREAKDOWN = 3
SQ_DEVICE_TIMEOUT = 4
SQ_CUDA_ERROR = 5
SQ_CAPACITY = 6
STATUS_NAMES = {0: "SQ_OK", 1: "SQ_BAD_INPUT", 2: "SQ_NO_CONVERGENCE", 3: "SQ_LANCZOS_BREAKDOWN",
                4: "SQ_DEVICE_TIMEOUT", 5: "SQ_CUDA_ERROR", 6: "SQ_CAPACITY"}

# every function the header declares, with its ctypes signature
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_l = ctypes.c_long
_d = ctypes.c_double
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)


class SqOptions(ctypes.Structure):
    _fields_ = [("faithful", ctypes.c_int), ("precision", ctypes.c_int), ("device", ctypes.c_int),
                ("list_format", ctypes.c_int), ("kernel", ctypes.c_int), ("tile", ctypes.c_int)]


class SqInfo(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int * 3), ("cube", ctypes.c_int * 3), ("n_qp", ctypes.c_int),
                ("fd_half_order", ctypes.c_int), ("bc", ctypes.c_int), ("n_atoms", ctypes.c_int),
                ("n_types", ctypes.c_int), ("n_images", ctypes.c_int),
                ("n_tables", ctypes.c_int), ("max_images_per_node", ctypes.c_int),
                ("precision", ctypes.c_int), ("faithful", ctypes.c_int), ("n_nodes", ctypes.c_long),
                ("h", ctypes.c_double * 3), ("cell_half", ctypes.c_double * 3),
                ("rcut", ctypes.c_double), ("beta", ctypes.c_double), ("dV", ctypes.c_double),
                ("n_electrons", ctypes.c_double), ("n_lm", ctypes.c_int),
                ("proj_points_per_node", ctypes.c_double), ("kernel_layout", ctypes.c_int),
                ("kernel_u_on_chip", ctypes.c_int), ("kernel_threads", ctypes.c_int),
                ("kernel_smem_bytes", ctypes.c_int)]


class SqPsdDesc(ctypes.Structure):
    _fields_ = [("n_r", ctypes.c_int), ("r", _dp), ("lmax", ctypes.c_int), ("lloc", ctypes.c_int),
                ("valence", ctypes.c_int), ("V", _dp * 4), ("U", _dp * 4),
                ("rc", ctypes.c_double * 4), ("rho_atom", _dp)]


class SqSystemDesc(ctypes.Structure):
    _fields_ = [("fd_order", ctypes.c_int), ("bc", ctypes.c_int),
                ("cell_half", ctypes.c_double * 3), ("grid", ctypes.c_int * 3),
                ("beta", ctypes.c_double), ("rcut", ctypes.c_double), ("n_qp", ctypes.c_int),
                ("n_types", ctypes.c_int), ("psd", ctypes.POINTER(SqPsdDesc)),
                ("n_atoms", ctypes.c_int), ("atom_type", _ip), ("atom_xyz", _dp),
                ("mixing_parameter", ctypes.c_double), ("mixing_history", ctypes.c_int),
                ("pulay_frequency", ctypes.c_int), ("tol_scf", ctypes.c_double),
                ("maxit_scf", ctypes.c_int), ("reference_cutoff", ctypes.c_double)]


class SqScfOptions(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("maxit", ctypes.c_int),
                ("mixing_parameter", ctypes.c_double), ("mixing_history", ctypes.c_int),
                ("pulay_frequency", ctypes.c_int), ("fermi_tol", ctypes.c_double),
                ("kerker_ktf", ctypes.c_double), ("cuda_graph", ctypes.c_int),
                ("learned_highpass", ctypes.c_double)]


class SqScfResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("free_energy", "free_energy_per_atom", "e_band", "e_xc",
                                       "e_xc_dc", "e_electrostatic", "e_self", "e_corr", "ts",
                                       "lambda_f", "residual", "seconds", "sq_ms", "tol")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


SIGNATURES = {
    "sq_create_from_deck": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p,
                                           ctypes.POINTER(SqOptions), ctypes.POINTER(_vp)]),
    "sq_destroy": (None, [_vp]),
    "sq_create": (ctypes.c_int, [ctypes.POINTER(SqSystemDesc), ctypes.POINTER(SqOptions),
                                 ctypes.POINTER(_vp)]),
    "sq_describe_system": (ctypes.c_int, [ctypes.POINTER(SqSystemDesc), ctypes.c_int,
                                          ctypes.POINTER(SqInfo), _dp, _dp]),
    "sq_describe_deck": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                        ctypes.POINTER(SqInfo), _dp, _dp]),
    "sq_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(SqInfo)]),
    "sq_plan_kernel": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(SqOptions),
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(SqInfo)]),
    "sq_nodes_and_weights": (ctypes.c_int, [_vp, _dp, _d, _l, _l, _dp, _dp, _dp, _dp]),
    "sq_nodes_and_weights_device": (ctypes.c_int, [_vp, _vp, _d, _l, _l, _vp, _vp, _vp, _vp, _vp]),
    "sq_sync_status": (ctypes.c_int, [_vp, _vp]),
    "sq_copy_lanczos_coefficients": (ctypes.c_int, [_vp, _dp, _dp, _l]),
    "sq_fermi_density_energy": (ctypes.c_int, [_vp, _dp, _dp, _l, _d, _d, _dp, _dp, _dp, _dp]),
    "sq_fermi_density_energy_device": (ctypes.c_int, [_vp, _vp, _vp, _l, _d, _d, _dp, _vp, _dp,
                                                      _dp, _vp]),
    "sq_electron_count_device": (ctypes.c_int, [_vp, _vp, _vp, _l, _d, _dp, _vp]),
    "sq_last_kernel_times": (ctypes.c_int, [_vp, _dp]),
    "sq_fermi_density_energy_noalloc": (ctypes.c_int, [_vp, _vp, _l, ctypes.c_int, _d, _d, _d,
                                                       _d, ctypes.c_int, _vp, _dp, _vp]),
    "sq_measure_fp32_peak": (ctypes.c_int, [ctypes.c_int, _dp]),
    "sq_tridiag_nodes_and_weights": (ctypes.c_int, [_dp, _dp, _l, ctypes.c_int, _dp, _dp, _dp,
                                                    _dp, ctypes.c_int]),
    "sq_fermi_timeout_selftest": (ctypes.c_int, [ctypes.c_int]),
    "sq_scf_shard_sq": (ctypes.c_int, [_vp, _l, _l, _dp]),
    "sq_scf_shard_counts": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "sq_scf_shard_density": (ctypes.c_int, [_vp, ctypes.c_double, _dp, _dp]),
    "sq_scf_shard_finish": (ctypes.c_int, [_vp, _dp, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.POINTER(SqScfResult)]),
    "sq_scf_begin": (ctypes.c_int, [_vp, ctypes.POINTER(SqScfOptions), _dp]),
    "sq_scf_begin_device": (ctypes.c_int, [_vp, ctypes.POINTER(SqScfOptions), _vp]),
    "sq_scf_step": (ctypes.c_int, [_vp, ctypes.POINTER(SqScfResult)]),
    "sq_scf_run": (ctypes.c_int, [_vp, ctypes.POINTER(SqScfOptions), _dp,
                                  ctypes.POINTER(SqScfResult)]),
    "sq_scf_get_density": (ctypes.c_int, [_vp, _dp, _dp]),
    "sq_scf_get_fields": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "sq_scf_history": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, ctypes.POINTER(ctypes.c_int)]),
    "sq_lda_pw92": (ctypes.c_int, [_dp, _l, _dp, _dp]),
    "sq_write_density_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _ip, _ip, _dp]),
    "sq_read_density_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _ip, _ip, _dp]),
    "sq_write_lambda_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _ip, _ip, _dp, _dp]),
    "sq_read_lambda_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _ip, _ip, _dp, _dp]),
    "sq_write_output_echo": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "sq_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(_vp)]),
    "sq_mlp_destroy": (None, [_vp]),
    "sq_mlp_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "sq_mlp_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_vp)]),
    "sq_mlp_set_params": (ctypes.c_int, [_vp, _fp, _fp, _fp, _d, _d]),
    "sq_mlp_get_params": (ctypes.c_int, [_vp, _fp, _fp, _fp, _dp, _dp]),
    "sq_descriptors": (ctypes.c_int, [_vp, _fp]),
    "sq_mlp_add_training_cell": (ctypes.c_int, [_vp, _vp]),
    "sq_mlp_train": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _d, _dp]),
    "sq_mlp_gradients": (ctypes.c_int, [_vp, _fp, _fp, _l, _dp, _fp]),
    "sq_mlp_forward": (ctypes.c_int, [_vp, _fp, _l, _fp]),
    "sq_mlp_predict_density": (ctypes.c_int, [_vp, _vp, _dp]),
    "sq_scf_begin_learned": (ctypes.c_int, [_vp, ctypes.POINTER(SqScfOptions), _vp]),
    "sq_batch_nodes_and_weights": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int,
                                                  ctypes.POINTER(_vp), _dp, ctypes.POINTER(_vp),
                                                  ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                                  ctypes.POINTER(_vp), _vp]),
    "sq_describe_scf_fields": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _dp, _dp, _dp,
                                              _dp]),
    "sq_last_error_string": (ctypes.c_char_p, []),
}

_lib = None


class SqError(RuntimeError):
    def __init__(self, status, where, msg):
        super().__init__("%s failed: %s (%s)" % (where, STATUS_NAMES.get(status, status), msg))
        self.status = status


def library_path():
    return _LIB


def lib():
    """Load the CUDA library; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise ImportError("sqminiapp_gb300 native library missing (%s); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`" % _LIB)
        L = ctypes.CDLL(_LIB)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, where):
    if status != SQ_OK:
        raise SqError(status, where, lib().sq_last_error_string().decode())
