"""FP64 numpy restatement of the SCF closure around the oracle's per-node SQ pass.

TEST INFRASTRUCTURE ONLY: tests/ and bench.py's CPU legs use it as the checker of the GPU SCF
(sq_scf_* in the product library); the product never imports it.

The reference declares the SCF driver and its pieces but gives them no bodies (SCF_LSSGQ,
src/lsdft.h:153; SolvePoisson :93; mix :183; Vxc_Calc_CA_PW / Exc_Calc_CA_PW :201-202;
SystemEnergy_Calc_lssgq :209; Generate_pseudocharge / PseudopotReference :217-218; the energy
fields Eself, Eself_TM, Ecorrection of src/ilsdft.h:149-155).  This module states the
published method those declarations name, independently of the CUDA implementation:

* pseudocharges b_J = -(1/4pi) Lap_FD V_loc,J on the box of the reference's pseudocharge
  cutoff (src/lsdft_initObjs.cc:628-817), V_loc sampled at the exact atom position;
* self energy E_self = 1/2 sum_J int b_J V_J (one image per atom) and the overlap correction
  E_c = 1/2 int (b_ref + b) V_c + E_self - E_self,ref, V_c = sum_J (V_ref,J - V_J), with the
  reference potential of Ghosh and Suryanarayana (SPARC) and REFERENCE_CUTOFF
  (src/lsdft_readfiles.cc:80,225);
* the atomic-superposition start density from the psd valence charge
  (src/lsdft_readfiles.cc:1033-1039), scaled to the electron count;
* the periodic Poisson problem -(1/4pi) Lap_FD phi = rho + b of the FD operator of
  Create_Laplacian (src/lsdft_initObjs.cc:308-367), solved exactly in Fourier space;
* LDA: Slater exchange + Perdew-Wang 1992 correlation (EXCHANGE_CORRELATION LDA_PW);
* Harris-Foulkes free energy and Periodic-Pulay mixing (Banerjee, Suryanarayana, Pask 2016)
  with MIXING_PARAMETER / MIXING_HISTORY / PULAY_FREQUENCY (src/lsdft_readfiles.cc:219-228).
"""
import math

import numpy as np

from . import Oracle, fermi_density_energy, spline


def round_half_away(v):
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def reference_potential(r, rc, z):
    """-z/r beyond rc; inside, -z/rc (9R^7 - 30R^6 + 28R^5 - 14R^2 + 12)/5 with R = r/rc."""
    r = np.asarray(r, dtype=np.float64)
    R = r / rc
    inner = -z / rc * (9 * R ** 7 - 30 * R ** 6 + 28 * R ** 5 - 14 * R ** 2 + 12) / 5
    with np.errstate(divide="ignore"):
        outer = -z / np.where(r > 0, r, 1.0)
    return np.where(r < rc, inner, outer)


def lda_pw92(rho):
    """(eps_xc, v_xc) of the unpolarised LDA: Slater exchange and the Perdew-Wang 1992
    correlation (Phys. Rev. B 45, 13244, Table I, zeta = 0); zero where rho <= 0."""
    rho = np.asarray(rho, dtype=np.float64)
    pos = rho > 0
    r = np.where(pos, rho, 1.0)
    A, a1, b1, b2, b3, b4 = 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294
    ex = -0.75 * (3.0 * r / math.pi) ** (1.0 / 3.0)
    rs = (3.0 / (4.0 * math.pi * r)) ** (1.0 / 3.0)
    q0 = -2 * A * (1 + a1 * rs)
    q1 = 2 * A * (b1 * np.sqrt(rs) + b2 * rs + b3 * rs ** 1.5 + b4 * rs ** 2)
    dq1 = A * (b1 / np.sqrt(rs) + 2 * b2 + 3 * b3 * np.sqrt(rs) + 4 * b4 * rs)
    lg = np.log1p(1.0 / q1)
    ec = q0 * lg
    dec = -2 * A * a1 * lg - q0 * dq1 / (q1 * q1 + q1)
    eps = np.where(pos, ex + ec, 0.0)
    v = np.where(pos, 4.0 / 3.0 * ex + ec - rs / 3.0 * dec, 0.0)
    return eps, v


def _stencil(V, c, o):
    """(1/2pi) times the -1/2 Laplacian stencil applied to the interior of V (z, y, x axes),
    i.e. -(1/4pi) Lap_FD V, on V[o:-o, o:-o, o:-o]."""
    cx, cy, cz = c
    core = V[o:-o, o:-o, o:-o]
    out = (cx[0] + cy[0] + cz[0]) * core
    nz, ny, nx = core.shape
    for q in range(1, o + 1):
        out = out + cx[q] * (V[o:-o, o:-o, o - q:o - q + nx] + V[o:-o, o:-o, o + q:o + q + nx])
        out = out + cy[q] * (V[o:-o, o - q:o - q + ny, o:-o] + V[o:-o, o + q:o + q + ny, o:-o])
        out = out + cz[q] * (V[o - q:o - q + nz, o:-o, o:-o] + V[o + q:o + q + nz, o:-o, o:-o])
    return out / (2 * math.pi)


def scf_fields(o: Oracle, reference_cutoff=0.5):
    """Pseudocharges, correction potential, start density, self energies and Poisson symbol
    of the oracle's deck; arrays are [nz, ny, nx] (x fastest, the node order)."""
    nx, ny, nz = o.grid
    N = np.array([nx, ny, nz])
    h = np.array(o.h)
    half = np.array(o.range)
    L = 2 * half
    order = o.order
    c = o.fd_coeffs()
    cut = o.pseudocharge_cutoff()
    pos, typ = o.atoms()
    shape = (nz, ny, nx)
    b = np.zeros(shape)
    bref = np.zeros(shape)
    vc = np.zeros(shape)
    rho = np.zeros(shape)
    e_self = 0.0
    e_self_ref = 0.0
    tables = []
    for t in range(o.ntype):
        r, vloc, rho_atom, z = o.psd_tables(t)
        rho_atom = rho_atom.copy()
        rho_atom[0] = rho_atom[1]
        peak = np.max(np.abs(rho_atom[1:]))
        big = np.nonzero(np.abs(rho_atom[1:]) > 1e-10 * peak)[0]
        rmax = min(float(r[1:][big[-1]]), 20.0)
        nb = np.rint(cut[t] / h).astype(int)
        nr = np.ceil(rmax / h).astype(int) + 1
        tables.append((r, vloc, rho_atom, z, rmax, nb, nr))

    def vloc_of(tab, rr):
        r, vloc, _, z, *_ = tab
        out = np.empty_like(rr)
        inside = rr <= r[-1]
        out[inside] = spline(r, vloc, rr[inside])
        out[~inside] = -z / rr[~inside]
        return out

    for n in range(o.natoms):
        tab = tables[typ[n]]
        r_t, _, rho_t, z, rmax, nb, nr = tab
        pmax = np.ceil(np.maximum(nb + order, nr) * h / L).astype(int) + 1
        for P in range(-pmax[0], pmax[0] + 1):
            for Q in range(-pmax[1], pmax[1] + 1):
                for R in range(-pmax[2], pmax[2] + 1):
                    home = P == 0 and Q == 0 and R == 0
                    x0 = pos[n] + np.array([P, Q, R]) * L
                    cen = round_half_away((x0 + half) / h).astype(int)
                    meets_b = np.all(cen + nb >= 0) and np.all(cen - nb <= N - 1)
                    meets_r = np.all(cen + nr >= 0) and np.all(cen - nr <= N - 1)
                    if meets_b or home:
                        ax = [h[a] * np.arange(cen[a] - nb[a] - order, cen[a] + nb[a] + order + 1)
                              - half[a] - x0[a] for a in range(3)]
                        Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
                        rr = np.sqrt(X * X + Y * Y + Z * Z)
                        V = vloc_of(tab, rr.ravel()).reshape(rr.shape)
                        Vr = reference_potential(rr, reference_cutoff, z)
                        bj = _stencil(V, c, order)
                        brj = _stencil(Vr, c, order)
                        Vi = V[order:-order, order:-order, order:-order]
                        Vri = Vr[order:-order, order:-order, order:-order]
                        if home:
                            e_self += 0.5 * np.sum(bj * Vi) * o.dV
                            e_self_ref += 0.5 * np.sum(brj * Vri) * o.dV
                        lo = cen - nb
                        sl_cell, sl_box = [], []
                        for a in range(3):
                            g0, g1 = max(lo[a], 0), min(lo[a] + 2 * nb[a] + 1, N[a])
                            sl_cell.append(slice(g0, g1))
                            sl_box.append(slice(g0 - lo[a], g1 - lo[a]))
                        if all(s.stop > s.start for s in sl_cell):
                            ci = (sl_cell[2], sl_cell[1], sl_cell[0])
                            bi = (sl_box[2], sl_box[1], sl_box[0])
                            b[ci] += bj[bi]
                            bref[ci] += brj[bi]
                            vc[ci] += (Vri - Vi)[bi]
                    if meets_r:
                        lo = np.maximum(cen - nr, 0)
                        hi = np.minimum(cen + nr, N - 1)
                        ax = [h[a] * np.arange(lo[a], hi[a] + 1) - half[a] - x0[a] for a in range(3)]
                        Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
                        rr = np.sqrt(X * X + Y * Y + Z * Z)
                        inside = rr <= rmax
                        vals = np.zeros(rr.shape)
                        vals[inside] = spline(r_t, rho_t, rr[inside])
                        rho[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] += vals
    e_corr = 0.5 * np.sum((bref + b) * vc) * o.dV + e_self - e_self_ref
    rho0 = np.maximum(rho * (o.n_electrons / (np.sum(rho) * o.dV)), 0.0)
    # Fourier symbol of the -1/2 Laplacian stencil per axis, then G = 2 pi / s on the R2C grid
    sym = []
    for a, cc in enumerate(c):
        m = np.arange(N[a])
        q = np.arange(1, order + 1)
        sym.append(cc[0] + 2 * np.sum(cc[1:, None] * np.cos(2 * math.pi * np.outer(q, m) / N[a]), axis=0))
    s = sym[2][:, None, None] + sym[1][None, :, None] + sym[0][None, None, :nx // 2 + 1]
    s[0, 0, 0] = 1.0
    green = 2 * math.pi / s
    green[0, 0, 0] = 0.0
    return {"b": b, "b_ref": bref, "vc": vc, "rho0": rho0, "green": green, "e_self": e_self,
            "e_self_ref": e_self_ref, "e_corr": e_corr, "b_total": float(np.sum(b) * o.dV)}


def poisson(rho_plus_b, green):
    """phi with -(1/4pi) Lap_FD phi = rho + b - mean (periodic, exact for the FD operator)."""
    return np.fft.irfftn(np.fft.rfftn(rho_plus_b) * green, s=rho_plus_b.shape, axes=(0, 1, 2))


def kerker(green, k_tf):
    """Kerker preconditioner k^2 / (k^2 + k_TF^2) with the FD symbol (k^2 -> 2 s(k) =
    4 pi / G(k)) on the R2C grid; 0 at k = 0 (the mean of a residual is dropped)."""
    with np.errstate(divide="ignore"):
        p = 4 * math.pi / (4 * math.pi + k_tf * k_tf * green)
    p[0, 0, 0] = 0.0
    return p


def periodic_pulay_step(x, f, state, k, mix, history, every, precond=None):
    """Next input density from x_k, f_k = rho_out - rho_in (Banerjee, Suryanarayana and Pask,
    Chem. Phys. Lett. 647 (2016) 31): x_{k+1} = xbar + mix P fbar with xbar = x - dX g,
    fbar = f - dF g, g = (dF^T dF)^-1 dF^T f when (k+1) % every == 0 (g = 0 otherwise), and P
    the Kerker preconditioner (precond = its R2C symbol) or the identity; negatives cut (the
    caller rescales to the electron count)."""
    if state.get("x_prev") is not None:
        state["dX"].append(x - state["x_prev"])
        state["dF"].append(f - state["f_prev"])
        state["dX"] = state["dX"][-history:]
        state["dF"] = state["dF"][-history:]
    state["x_prev"], state["f_prev"] = x.copy(), f.copy()
    xbar, fbar = x, f
    if (k + 1) % every == 0 and state["dF"]:
        F = np.stack([d.ravel() for d in state["dF"]], axis=1)
        X = np.stack([d.ravel() for d in state["dX"]], axis=1)
        A = F.T @ F
        d = 1.0 / np.sqrt(np.diag(A))
        As = A * d[:, None] * d[None, :]
        try:
            g = np.linalg.solve(As, (F.T @ f.ravel()) * d) * d
            xbar = (x.ravel() - X @ g).reshape(x.shape)
            fbar = (f.ravel() - F @ g).reshape(x.shape)
        except np.linalg.LinAlgError:
            pass
    if precond is not None:
        fbar = np.fft.irfftn(np.fft.rfftn(fbar) * precond, s=fbar.shape, axes=(0, 1, 2))
    return np.maximum(xbar + mix * fbar, 0.0)


def scf(o: Oracle, fields=None, tol=1e-6, maxit=100, mix=0.3, history=7, pulay_every=2,
        rho_init=None, nthreads=None, fermi_tol=1e-12, k_tf=1.0):
    """SCF with the oracle's per-node Lanczos/quadrature (corrected operator expected).
    k_tf > 0: Kerker-preconditioned mixing with that Thomas-Fermi wave vector (1/bohr);
    k_tf <= 0: unpreconditioned.  Returns the last iteration's quantities and the history of
    free energy and residual."""
    if fields is None:
        fields = scf_fields(o)
    shape = fields["b"].shape
    dV = o.dV
    ne = o.n_electrons
    x = fields["rho0"].copy() if rho_init is None else np.maximum(np.reshape(rho_init, shape), 0.0)
    x *= ne / (np.sum(x) * dV)
    state = {"dX": [], "dF": [], "x_prev": None}
    pk = kerker(fields["green"], k_tf) if k_tf > 0 else None
    hist_F, hist_err = [], []
    out = {}
    for k in range(maxit):
        phi = poisson(x + fields["b"], fields["green"])
        eps, vxc = lda_pw92(x)
        veff = phi + vxc
        q = o.nodes_and_weights(veff=veff.ravel(), veff_const=0.0, nthreads=nthreads)
        fr = fermi_density_energy(q["lambda"], q["weights"], o.beta, ne, dV, tol=fermi_tol,
                                  maxit=400)
        rho_out = fr["rho"].reshape(shape)
        e_xc = np.sum(x * eps) * dV
        e_xc_dc = np.sum(x * vxc) * dV
        e_es = 0.5 * np.sum((fields["b"] - x) * phi) * dV
        F = (fr["e_band"] + e_xc - e_xc_dc + e_es - fields["e_self"] + fields["e_corr"]
             + fr["ts"])
        f = rho_out - x
        err = float(np.linalg.norm(f) / np.linalg.norm(rho_out))
        hist_F.append(F)
        hist_err.append(err)
        out = {"iterations": k + 1, "free_energy": F, "free_energy_per_atom": F / o.natoms,
               "e_band": fr["e_band"], "e_xc": e_xc, "e_xc_dc": e_xc_dc, "e_electrostatic": e_es,
               "e_self": fields["e_self"], "e_corr": fields["e_corr"], "ts": fr["ts"],
               "lambda_f": fr["lambda_f"], "residual": err, "rho_out": rho_out, "rho_in": x,
               "phi": phi, "vxc": vxc, "converged": err < tol}
        if err < tol:
            break
        x = periodic_pulay_step(x, f, state, k, mix, history, pulay_every, pk)
        x *= ne / (np.sum(x) * dV)
    out["free_energy_history"] = np.array(hist_F)
    out["residual_history"] = np.array(hist_err)
    return out
