"""The mixed form's table rebuild on the tensor cores: M = Phi lambda (and
Phi lambda^T for the down spin), formed by the split-bf16 tcgen05 GEMM with
exact FP32 slice sums, against the same product in FP64 (torch) from the
library's FP64 AO values.  The bar is 1e-11 of sum_a |Phi_a| |lambda_ab| per
entry: six 8-bit slices carry 47 bits of each operand row or column, the slice
levels 0-2 sum exactly and levels 3-5 round toward zero in FP32 (about 2^-40);
the rebuild's G and G^-1 then agree with the FP64 form (test_gpu_mixed.py), and
the tensor-core rebuild replaces the geminal assembly of
jqmc/determinant.py:1380-1402."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _without_j3(ham):
    """The Hamiltonian without its three-body Jastrow: M depends on the geminal
    alone, and without J3 the build leaves M in the rebuild scratch (the J3
    field's work space overwrites it otherwise)."""
    from dataclasses import replace
    wf = ham.wavefunction_data
    jd = replace(wf.jastrow_data, jastrow_three_body_data=None)
    return replace(ham, wavefunction_data=replace(wf, jastrow_data=jd))


@pytest.mark.parametrize("name,walkers", [("water_like", 8), ("ring12", 40), ("chain32", 6)])
def test_tensor_core_lambda_gemm_matches_fp64(name, walkers):
    from jqmc_gb300 import _lib, synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    syn = synthetic.SYSTEMS[name]()
    gs = GpuSystem(_without_j3(syn.hamiltonian))
    assert _lib.lib().jqmc_tensor_core_rebuild(gs.handle) == 1
    n, A = gs.n_up, gs.A
    r_up, r_dn = syn.initial_electrons(walkers, seed=5)
    ws = WalkerSet(gs, r_up, r_dn, precision="mixed")   # the build forms M in the scratch
    torch.cuda.synchronize()
    pairs = ws.scratch.view(torch.float32).view(walkers, 2, n, A, 2).double()
    m = pairs[..., 0] + pairs[..., 1]                  # slot 0: M_dn = Phi_dn lambda^T, slot 1: M_up = Phi_up lambda
    lam = torch.as_tensor(gs._keep["lam"], device=gs.device)
    for slot, r, L in ((1, r_up, lam), (0, r_dn, lam.T)):
        pts = torch.as_tensor(np.asarray(r).reshape(-1, 3), device=gs.device)
        phi = gs.ao_vgl(pts)[0].T.contiguous()          # (walkers * n, A), FP64
        ref = (phi @ L).view(walkers, n, A)
        scale = (phi.abs() @ L.abs()).view(walkers, n, A)
        err = float(((m[:, slot] - ref).abs() / scale).max())
        print(f"{name} slot {slot}: max error {err:.2e} of sum |Phi||lambda|")
        assert err < 1e-11, (name, slot, err)
    assert not ws.status.any()


def test_tensor_core_rebuild_twice_is_identical():
    """Two builds of the same walkers (the workspace reused, the second one
    smaller) give bit-identical tables."""
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    syn = synthetic.ring12()
    gs = GpuSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(300, seed=9)
    a = WalkerSet(gs, r_up, r_dn, precision="mixed")
    b = WalkerSet(gs, r_up[:100], r_dn[:100], precision="mixed")
    torch.cuda.synchronize()
    assert torch.equal(a.Tup[:100], b.Tup) and torch.equal(a.Ginv[:100], b.Ginv)
