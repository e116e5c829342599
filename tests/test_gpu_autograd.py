"""The likelihood as a PyTorch autograd operation: values and gradients equal the
engine's host results; the backward pass weights each instance's gradient by the
incoming gradient of its log-likelihood."""
import numpy as np
import pytest

from gpu_cases import random_instance

import mcphylo_gb300 as mp

pytestmark = pytest.mark.gpu


def _engine(insts, precision):
    e = mp.Engine(insts[0].K, len(insts[0].rates), precision, n_instances=len(insts))
    for i, b in enumerate(insts):
        e.set_tree(b.parent, b.blen, i)
        e.set_codes(b.codes, b.leaf_nums, i)
        e.set_model(b.U, b.D, b.Uinv, b.mu, b.pi, b.rates, i)
    return e


@pytest.mark.parametrize("side_stream", [False, True])
def test_autograd_matches_engine(built_lib, side_stream):
    import torch
    from mcphylo_gb300.autograd import phylo_loglik
    insts = [random_instance(4, 2, 12, 150, seed=81), random_instance(4, 2, 20, 90, seed=82)]
    e = _engine(insts, "f64")
    host = _engine(insts, "f64")
    off = e.grad_offsets()
    rng = np.random.default_rng(3)
    b = np.concatenate([x.blen for x in insts]) * rng.uniform(0.8, 1.2, int(off[-1]))
    host.set_all_branch_lengths(b)
    ll_h, g_h = host.logpdf_grad()
    stream = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        blen = torch.tensor(b, dtype=torch.float64, device="cuda", requires_grad=True)
        ll = phylo_loglik(e, blen)
        w = torch.tensor([1.0, -2.5], dtype=torch.float64, device="cuda")
        (ll * w).sum().backward()
    torch.cuda.synchronize()
    np.testing.assert_allclose(ll.detach().cpu().numpy(), ll_h, rtol=1e-13)
    want = np.concatenate([g_h[off[0]:off[1]] * 1.0, g_h[off[1]:off[2]] * -2.5])
    np.testing.assert_allclose(blen.grad.cpu().numpy(), want, rtol=1e-12, atol=1e-12)


def test_autograd_checks_its_input(built_lib):
    import torch
    from mcphylo_gb300.autograd import phylo_loglik
    inst = random_instance(4, 1, 8, 40, seed=83)
    e = _engine([inst], "f32")
    with pytest.raises(ValueError):
        phylo_loglik(e, torch.ones(3, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        phylo_loglik(e, torch.ones(len(inst.blen), dtype=torch.float32, device="cuda"))
