"""ctypes binding of the FP64 CPU oracle (oracle/sq_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the oracle restates the reference SQMiniApp per-node
Spectral Quadrature path (src/lsdft_scf.cc:32-164, src/lsdft_matvec.cc:25-149,
src/lsdft_nl.cc:6-208, src/lsdft_tools.cc:15-151,156-370,912-1026,
src/lsdft_initObjs.cc:393-475,576-967,1409-1946,2612-2663,
src/lsdft_readfiles.cc:21-497,677-1101) in FP64 on the CPU.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU legs use it, always as the checker
or the timed CPU baseline, never as part of the product path.

Parity unpinned: the reference prints no lambda/weight values and needs PETSc
and MPI to build, so the oracle is pinned by the counts in the reference's run
logs and by independent mathematical known-answer tests instead.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "libsq_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build(force=False):
    """Compile the oracle with make (g++, no GPU needed)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.sqo_open.restype = ctypes.c_void_p
        L.sqo_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
                               ctypes.c_int]
        L.sqo_close.argtypes = [ctypes.c_void_p]
        L.sqo_dims.argtypes = [ctypes.c_void_p, _ip, _dp]
        L.sqo_fd_coeffs.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.sqo_gamma.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.sqo_pseudocharge_cutoff.argtypes = [ctypes.c_void_p, _dp]
        L.sqo_local_overlap_count.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 6 + [_dp, _ip]
        L.sqo_nodes_and_weights.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, _lp,
                                            ctypes.c_long, ctypes.c_int, _dp, _dp, _dp, _dp, _dp,
                                            _dp]
        L.sqo_matvec.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double, ctypes.c_long, _dp, _dp]
        L.sqo_ql.argtypes = [_dp, _dp, ctypes.c_int, _dp, _dp, _dp, _dp]
        L.sqo_fermi_density_energy.argtypes = [_dp, _dp, ctypes.c_long, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _dp,
                                               _ip]
        L.sqo_spline.argtypes = [_dp, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int]
        L.sqo_psd_tables.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp, _dp, _dp, _dp]
        L.sqo_atoms.argtypes = [ctypes.c_void_p, _dp, _ip]
        L.sqo_ylm.restype = ctypes.c_double
        L.sqo_ylm.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


class Oracle:
    """One deck opened in the oracle (FP64, CPU)."""

    def __init__(self, deck_dir, name, faithful=True):
        err = ctypes.create_string_buffer(512)
        self._h = lib().sqo_open(deck_dir.encode(), name.encode(), 1 if faithful else 0, err, 512)
        if not self._h:
            raise RuntimeError("oracle: " + err.value.decode())
        ints = np.zeros(16, np.int32)
        dbls = np.zeros(16, np.float64)
        lib().sqo_dims(self._h, ints.ctypes.data_as(_ip), _d(dbls))
        self.grid = tuple(int(v) for v in ints[0:3])
        self.nloc = tuple(int(v) for v in ints[3:6])
        self.n_qp = int(ints[6])
        self.n_nodes = int(ints[7])
        self.ntype = int(ints[8])
        self.natoms = int(ints[9])
        self.n_images = int(ints[10])
        self.order = int(ints[11])
        self.bc = int(ints[12])
        self.nlm0 = int(ints[13])
        self.n_electrons = int(ints[14])
        self.faithful = bool(ints[15])
        self.h = tuple(float(v) for v in dbls[0:3])
        self.range = tuple(float(v) for v in dbls[3:6])
        self.rcut = float(dbls[6])
        self.beta = float(dbls[7])
        self.dV = float(dbls[8])

    def close(self):
        if self._h:
            lib().sqo_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fd_coeffs(self):
        c = [np.zeros(self.order + 1) for _ in range(3)]
        lib().sqo_fd_coeffs(self._h, _d(c[0]), _d(c[1]), _d(c[2]))
        return c

    def gamma(self, t=0):
        g = np.zeros(4)
        lib().sqo_gamma(self._h, t, _d(g))
        return g

    def pseudocharge_cutoff(self):
        c = np.zeros(3 * self.ntype)
        lib().sqo_pseudocharge_cutoff(self._h, _d(c))
        return c.reshape(self.ntype, 3)

    def psd_tables(self, t=0):
        """(r, V_loc, rho_atom, z_valence) of type t as read from its psd file."""
        n = ctypes.c_int(0)
        lib().sqo_psd_tables(self._h, t, ctypes.byref(n), None, None, None, None)
        r, v, rho = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        z = ctypes.c_double(0)
        lib().sqo_psd_tables(self._h, t, ctypes.byref(n), _d(r), _d(v), _d(rho), ctypes.byref(z))
        return r, v, rho, z.value

    def atoms(self):
        """(positions [natoms, 3], types [natoms]) in .ion order."""
        pos = np.zeros((self.natoms, 3))
        typ = np.zeros(self.natoms, np.int32)
        lib().sqo_atoms(self._h, _d(pos), typ.ctypes.data_as(_ip))
        return pos, typ

    def local_overlap_count(self, cor, dims, extra_xyz=None):
        cnt = ctypes.c_int(0)
        ex = None if extra_xyz is None else np.asarray(extra_xyz, np.float64)
        lib().sqo_local_overlap_count(self._h, *[int(v) for v in cor], *[int(v) for v in dims],
                                      _d(ex), ctypes.byref(cnt))
        return cnt.value

    def nodes_and_weights(self, nodes=None, veff=None, veff_const=0.333, nthreads=None,
                          want_ab=False):
        if nodes is None:
            nodes = np.arange(self.n_nodes, dtype=np.int64)
        nodes = np.ascontiguousarray(nodes, dtype=np.int64)
        n = len(nodes)
        q = self.n_qp
        lam = np.zeros((n, q))
        w = np.zeros((n, q))
        lmin = np.zeros(n)
        lmax = np.zeros(n)
        a = np.zeros((n, q + 1)) if want_ab else None
        b = np.zeros((n, q + 1)) if want_ab else None
        if veff is not None:
            veff = np.ascontiguousarray(veff, dtype=np.float64)
            assert veff.size == self.n_nodes
        if nthreads is None:
            nthreads = os.cpu_count() or 1
        st = lib().sqo_nodes_and_weights(self._h, _d(veff), float(veff_const),
                                         nodes.ctypes.data_as(_lp), n, int(nthreads), _d(a),
                                         _d(b), _d(lam), _d(w), _d(lmin), _d(lmax))
        if st != 0:
            raise RuntimeError("oracle nodes_and_weights status %d" % st)
        out = {"lambda": lam, "weights": w, "lambda_min": lmin, "lambda_max": lmax}
        if want_ab:
            out["a"] = a
            out["b"] = b
        return out

    def matvec(self, node, x, veff=None, veff_const=0.333):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        if veff is not None:
            veff = np.ascontiguousarray(veff, dtype=np.float64)
        lib().sqo_matvec(self._h, _d(veff), float(veff_const), int(node), _d(x), _d(y))
        return y

    def dense_hamiltonian(self, node, veff=None, veff_const=0.333):
        n = self.nloc[0] * self.nloc[1] * self.nloc[2]
        H = np.zeros((n, n))
        e = np.zeros(n)
        for j in range(n):
            e[:] = 0.0
            e[j] = 1.0
            H[:, j] = self.matvec(node, e, veff, veff_const)
        return H


def ql(diag, sub):
    diag = np.ascontiguousarray(diag, dtype=np.float64)
    sub = np.ascontiguousarray(sub, dtype=np.float64)
    n = len(diag)
    lam = np.zeros(n)
    w = np.zeros(n)
    lo = ctypes.c_double()
    hi = ctypes.c_double()
    st = lib().sqo_ql(_d(diag), _d(sub), n, _d(lam), _d(w), ctypes.byref(lo), ctypes.byref(hi))
    if st != 0:
        raise RuntimeError("QL did not converge")
    return lam, w, lo.value, hi.value


def fermi_density_energy(lam, w, beta, n_electrons, dV, tol=1e-12, maxit=200):
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n_nodes, q = lam.shape
    rho = np.zeros(n_nodes)
    lf = ctypes.c_double()
    eb = ctypes.c_double()
    ts = ctypes.c_double()
    it = ctypes.c_int()
    lib().sqo_fermi_density_energy(_d(lam), _d(w), n_nodes, q, float(beta), float(n_electrons),
                                   float(dV), float(tol), int(maxit), ctypes.byref(lf), _d(rho),
                                   ctypes.byref(eb), ctypes.byref(ts), ctypes.byref(it))
    return {"lambda_f": lf.value, "rho": rho, "e_band": eb.value, "ts": ts.value,
            "iters": it.value}


def spline(x, y, xq):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    xq = np.ascontiguousarray(xq, dtype=np.float64)
    yq = np.zeros_like(xq)
    if lib().sqo_spline(_d(x), _d(y), len(x), _d(xq), _d(yq), len(xq)) != 0:
        raise RuntimeError("spline out of range")
    return yq


def ylm(x, y, z, l, m):
    return lib().sqo_ylm(float(x), float(y), float(z), int(l), int(m))
