"""Adjoint kernel (jqmc_dlnpsi_dparam) against the oracle's closed-form derivatives
(themselves pinned by finite differences in test_oracle_adjoint.py), and the
torch.autograd backward built on it.  FP64 bar: 1e-10 relative to the block's
largest magnitude."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=["water_like", "ring12"])
def setup(request):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[request.param]()
    gs = GpuSystem(syn.hamiltonian)
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(6, seed=41)
    ws = WalkerSet(gs, r_up, r_dn)
    return syn, gs, o, ws, r_up, r_dn


def test_dlnpsi_dparams_match_oracle(setup):
    from jqmc_gb300.adjoint import dlnpsi_dparams
    from oracle import adjoint as AD
    syn, gs, o, ws, r_up, r_dn = setup
    got = {k: v.cpu().numpy() for k, v in dlnpsi_dparams(ws).items()}
    assert set(got) == {"j1_param", "j2_param", "j3_matrix", "lambda_matrix"}
    for w in range(ws.nwalk):
        ref = AD.dlnpsi_dparams(o, r_up[w], r_dn[w])
        for k in ref:
            assert _rel(got[k][w], ref[k]) < RTOL, (k, w)


def test_lnpsi_autograd_backward(setup):
    from jqmc_gb300.adjoint import dlnpsi_dparams, ln_psi
    syn, gs, o, ws, r_up, r_dn = setup
    blocks = dlnpsi_dparams(ws)
    params = {k: torch.zeros(v.shape[1:], dtype=torch.float64, device=gs.device, requires_grad=True) for k, v in blocks.items()}
    out = ln_psi(ws, params)
    ld, _, jj = ws.log_psi()
    assert torch.allclose(out, ld + jj)
    g = torch.linspace(0.5, 1.5, ws.nwalk, dtype=torch.float64, device=gs.device)
    out.backward(g)
    for k, p in params.items():
        ref = torch.einsum("w,w...->...", g, blocks[k])
        assert _rel(p.grad.cpu().numpy(), ref.cpu().numpy()) < 1e-13, k
