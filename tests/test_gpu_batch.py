"""GPU mixed-cell batch: several independent cells (different meshes, cubes, Lanczos degrees
and precisions) in one sq_batch_nodes_and_weights submission give the results of one
sq_nodes_and_weights call per cell.

Tolerance: each node is computed by one CTA in either case; only the order of the atomic
accumulations inside a node can differ, so FP64 cells agree to 1e-10 and FP32 cells to 1e-4 on
the quadrature moments (the parity tolerances of the single-cell tests)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_single_cells(deck_dir, small_cell, tmp_path):
    import torch
    from sqminiapp_gb300 import LSDFT, batch_nodes_and_weights
    from sqminiapp_gb300.decks import make_fcc_mg_deck
    d2, n2, _ = make_fcc_mg_deck(str(tmp_path / "b"), "b", ncell=1, h=0.65, rcut=3.0, n_qp=14,
                                 disp=0.2, seed=31)
    cells = [LSDFT(*small_cell[:2], faithful=False, precision=64),
             LSDFT(deck_dir, "Mg1", faithful=False, precision=32),
             LSDFT(d2, n2, faithful=False, precision=32)]
    rng = np.random.default_rng(8)
    dev = torch.device("cuda", 0)
    veffs, outs, refs = [], [], []
    for e in cells:
        v = -0.2 + 0.05 * rng.standard_normal(e.n_nodes)
        refs.append(e.NodesAndWeights_LSSGQ(veff=v))
        veffs.append(torch.from_numpy(v).to(dev))
        outs.append({k: torch.empty(s, dtype=torch.float64, device=dev) for k, s in
                     (("lambda", (e.n_nodes, e.n_qp)), ("weights", (e.n_nodes, e.n_qp)),
                      ("lambda_min", (e.n_nodes,)), ("lambda_max", (e.n_nodes,)))})
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):  # twice in a row: the second split uses the measured node costs
        batch_nodes_and_weights(cells, [v.data_ptr() for v in veffs], None,
                                [{k: t.data_ptr() for k, t in o.items()} for o in outs], stream)
        torch.cuda.synchronize()
        for e, o, r in zip(cells, outs, refs):
            tol = 1e-10 if e.precision == 64 else 1e-4
            lam, w = o["lambda"].cpu().numpy(), o["weights"].cpu().numpy()
            for k in range(4):
                got = np.sum(w * lam ** k, axis=1)
                exp = np.sum(r["weights"] * r["lambda"] ** k, axis=1)
                assert np.max(np.abs(got - exp) / np.maximum(1.0, np.abs(exp))) < tol
    for e in cells:
        e.close()
