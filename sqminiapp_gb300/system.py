"""A cell in memory: the values the reference's input readers put into LSDFT_OBJ
(src/lsdft_readfiles.cc:21-1101), as numpy arrays, for sq_create (sq_system_desc).

read_system(deck_dir, name) reads a deck into that form with the conversions of the
reference's Read_Pseudopotential (V_l = value / (2 r), U_l = value / r, valence density
divided by 4 pi r^2, the r = 0 row copied from r[1]); to_desc() packs such a dict into the
C structs, keeping the arrays alive with the returned object.
"""
import ctypes
import math
import os

import numpy as np

from .capi import SqPsdDesc, SqSystemDesc

_DEFAULTS = {"mixing_parameter": 0.0, "mixing_history": 0, "pulay_frequency": 0, "tol_scf": 0.0,
             "maxit_scf": 0, "reference_cutoff": 0.0}


def _tokens(path):
    with open(path) as f:
        return f.read().split()


def _read_psd(path, type_name, lloc, valence):
    with open(path) as f:
        lines = f.read().splitlines()
    if not lines or lines[0].split()[0] != type_name:
        raise ValueError("%s: pseudopotential does not match atom type %s" % (path, type_name))
    sections = []
    for line in lines[1:]:
        t = line.strip()
        if "follows" in t:
            sections.append((t, []))
        elif sections:
            sections[-1][1].extend(float(x) for x in line.split())
    grid = [v for k, v in sections if k == "Radial grid follows"][0]
    nr = len(grid)
    r = np.concatenate([[0.0], grid])
    V = [None] * 4
    U = [None] * 4
    rc = [0.0] * 4
    rho = np.zeros(nr + 1)
    lmax = -1
    for key, v in sections:
        if key == "Pseudopotential follows (l on next line)":
            l = int(v[0])
            lmax = l
            V[l] = np.empty(nr + 1)
            V[l][1:] = 0.5 * np.asarray(v[1:nr + 1]) / r[1:]
            V[l][0] = V[l][1]
        elif key == "Valence charge follows":
            rho[1:] = np.asarray(v[:nr]) / (4 * math.pi * r[1:] ** 2)
        elif key == "Pseudo-wave-function follows (l, zelect, rc)":
            l = int(v[0])
            rc[l] = v[2]
            U[l] = np.empty(nr + 1)
            U[l][1:] = np.asarray(v[3:nr + 3]) / r[1:]
            U[l][0] = U[l][1]
    for l in range(4):
        if l != lloc and l <= lmax and U[l] is None:
            raise ValueError("%s: missing wave function for l=%d" % (path, l))
        if l == lloc:
            U[l] = None
    return {"r": r, "lmax": lmax, "lloc": lloc, "valence": valence, "V": V, "U": U, "rc": rc,
            "rho_atom": rho}


def read_system(deck_dir, name):
    """The cell of <deck_dir>/<name>.inpt/.ion and its pseudopotentials as a dict."""
    t = _tokens(os.path.join(deck_dir, name + ".inpt"))
    sysd = {"fd_order": 12, "bc": 1, "cell_half": None, "grid": None, "beta": 1000.0,
            "rcut": 12.0, "n_qp": 50}
    sysd.update(_DEFAULTS)
    lloc, files, i = None, None, 0
    keys = {"MIXING_PARAMETER:": ("mixing_parameter", float), "MIXING_HISTORY:": ("mixing_history", int),
            "PULAY_FREQUENCY:": ("pulay_frequency", int), "TOL_SCF:": ("tol_scf", float),
            "MAXIT_SCF:": ("maxit_scf", int), "REFERENCE_CUTOFF:": ("reference_cutoff", float),
            "BETA:": ("beta", float), "RADIUS_TRUNC:": ("rcut", float),
            "LANCZOS_DEGREE:": ("n_qp", int), "FD_ORDER:": ("fd_order", int),
            "BOUNDARY_CONDITION:": ("bc", int)}
    ntype = None
    while i < len(t):
        k = t[i]
        i += 1
        if k in keys:
            name_, typ = keys[k]
            sysd[name_] = typ(t[i])
            i += 1
        elif k == "CELL:":
            sysd["cell_half"] = [float(x) for x in t[i:i + 3]]
            i += 3
        elif k == "FD_GRID:":
            sysd["grid"] = [int(x) for x in t[i:i + 3]]
            i += 3
        elif k == "NTYPE:":
            ntype = int(t[i])
            i += 1
        elif k == "PSEUDOPOTENTIAL_LOCAL:":
            lloc = [int(x) for x in t[i:i + ntype]]
            i += ntype
        elif k == "PSEUDOPOTENTIAL_FILE:":
            files = t[i:i + ntype]
            i += ntype
    ion = _tokens(os.path.join(deck_dir, name + ".ion"))
    natoms, j = int(ion[0]), 1
    types, atom_type, xyz = [], [], []
    while j < len(ion):
        tname, ne, na = ion[j], int(ion[j + 1]), int(ion[j + 2])
        j += 3
        tt = len(types)
        types.append(_read_psd(os.path.join(deck_dir, "pseudopotential", files[tt]), tname,
                               lloc[tt], ne))
        for _ in range(na):
            xyz.append([float(x) for x in ion[j:j + 3]])
            atom_type.append(tt)
            j += 3
    assert len(atom_type) == natoms
    sysd["types"] = types
    sysd["atom_type"] = np.asarray(atom_type, dtype=np.int32)
    sysd["atom_xyz"] = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    return sysd


class _Packed:
    """The C description of a system dict plus the arrays it points into."""

    def __init__(self, sysd):
        dp = ctypes.POINTER(ctypes.c_double)
        self.keep = []

        def arr(a, dtype=np.float64):
            a = np.ascontiguousarray(a, dtype=dtype)
            self.keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(np.ctypeslib.as_ctypes_type(dtype)))

        psd = (SqPsdDesc * len(sysd["types"]))()
        for k, tp in enumerate(sysd["types"]):
            p = psd[k]
            p.n_r = len(tp["r"])
            p.r = arr(tp["r"])
            p.lmax, p.lloc, p.valence = tp["lmax"], tp["lloc"], tp["valence"]
            for l in range(4):
                p.V[l] = arr(tp["V"][l]) if tp["V"][l] is not None else dp()
                p.U[l] = arr(tp["U"][l]) if tp["U"][l] is not None else dp()
                p.rc[l] = tp["rc"][l]
            p.rho_atom = arr(tp["rho_atom"]) if tp.get("rho_atom") is not None else dp()
        self.psd = psd
        d = SqSystemDesc()
        d.fd_order, d.bc = sysd["fd_order"], sysd["bc"]
        d.cell_half[:] = sysd["cell_half"]
        d.grid[:] = sysd["grid"]
        d.beta, d.rcut, d.n_qp = sysd["beta"], sysd["rcut"], sysd["n_qp"]
        d.n_types = len(sysd["types"])
        d.psd = psd
        d.n_atoms = len(sysd["atom_type"])
        d.atom_type = arr(sysd["atom_type"], np.int32)
        d.atom_xyz = arr(np.asarray(sysd["atom_xyz"]).reshape(-1))
        for k in _DEFAULTS:
            setattr(d, k, sysd.get(k, _DEFAULTS[k]))
        self.desc = d


def to_desc(sysd):
    return _Packed(sysd)
