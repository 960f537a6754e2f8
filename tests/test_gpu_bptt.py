"""Differentiation form: the hand-written LIF BPTT kernels against an FP64 autograd reference and
against finite differences of the sigmoid-relaxed forward.

Tolerances. Hard-threshold forward (the trained form): relative L2 error of each weight gradient
below 1e-4 against FP64 autograd, with identical spike counts. Relaxed forward (the form whose exact
derivative the surrogate is): the problem is ill-conditioned in FP32 (slope-25 sigmoid through 32
recurrent steps; a plain PyTorch FP32 implementation is itself ~0.5% from FP64), so the kernels must
be as close to the FP64 answer as that FP32 implementation: error <= 2 x the FP32 implementation's
error + 1e-4 (relative L2) against FP64 autograd, and per entry against central finite differences
(step 1e-3, FP64): |kernel - fd| <= 2 |fp32 - fd| + 1e-3 |fd| + 1e-6.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _grads(model, x, labels):
    from knp_gb300 import bptt

    model.zero_grad(set_to_none=True)
    counts = model(x)
    loss = bptt.loss_fn(counts, labels)
    loss.backward()
    return counts.detach(), loss.detach(), [w.grad.detach().clone() for w in model.weights]


def _ref_grads(model, x, labels, relaxed, dtype=torch.float64):
    from knp_gb300 import bptt

    ws = [bptt.bf16_values(w.detach()).to(dtype).requires_grad_(True) for w in model.weights]
    counts = bptt.reference_forward(x.to(dtype), ws, model.beta, model.theta, relaxed, model.k)
    loss = torch.nn.functional.cross_entropy(counts, labels)
    loss.backward()
    return counts.detach(), loss.detach(), [w.grad.to(torch.float64) for w in ws]


def _rel(a, b):
    return (a.to(torch.float64) - b).norm().item() / max(b.norm().item(), 1e-30)


@pytest.mark.parametrize("relaxed", [False, True])
@pytest.mark.parametrize("checkpoint", [8, 5])
def test_bptt_matches_fp64_autograd(relaxed, checkpoint):
    from knp_gb300 import bptt

    x, labels = bptt.make_batch(T=32, B=16, seed=3)
    model = bptt.SpikingMLP(sizes=(784, 128, 64, 10), checkpoint=checkpoint, relaxed=relaxed, seed=1)
    counts, loss, grads = _grads(model, x, labels)
    rc, rl, rg = _ref_grads(model, x, labels, relaxed)
    if not relaxed:
        assert torch.equal(counts.to(torch.float64), rc)  # identical spike counts
        for g, r in zip(grads, rg):
            assert _rel(g, r) < 1e-4, _rel(g, r)
    else:
        _, _, r32 = _ref_grads(model, x, labels, relaxed, torch.float32)
        for g, r, f in zip(grads, rg, r32):
            assert _rel(g, r) <= 2 * _rel(f, r) + 1e-4, (_rel(g, r), _rel(f, r))


def test_bptt_finite_differences_relaxed():
    from knp_gb300 import bptt

    x, labels = bptt.make_batch(T=12, B=8, seed=5)
    model = bptt.SpikingMLP(sizes=(784, 64, 32, 10), checkpoint=4, relaxed=True, seed=2)
    _, _, grads = _grads(model, x, labels)
    _, _, g32 = _ref_grads(model, x, labels, True, torch.float32)
    ws64 = [bptt.bf16_values(w.detach()).to(torch.float64) for w in model.weights]

    def loss64(ws):
        c = bptt.reference_forward(x, ws, model.beta, model.theta, True, model.k)
        return torch.nn.functional.cross_entropy(c, labels).item()

    gen = torch.Generator().manual_seed(0)
    eps = 1e-3
    for li, w in enumerate(ws64):
        idx = torch.randint(0, w.numel(), (6,), generator=gen)
        fd = []
        for i in idx.tolist():
            wp = [v.clone() for v in ws64]
            wm = [v.clone() for v in ws64]
            wp[li].view(-1)[i] += eps
            wm[li].view(-1)[i] -= eps
            fd.append((loss64(wp) - loss64(wm)) / (2 * eps))
        fd = torch.tensor(fd, dtype=torch.float64)
        dev_idx = idx.to(grads[li].device)
        an = grads[li].view(-1)[dev_idx].to(torch.float64).cpu()
        f32 = g32[li].view(-1)[dev_idx].cpu()
        tol = 2 * (f32 - fd).abs() + 1e-3 * fd.abs() + 1e-6
        assert torch.all((an - fd).abs() <= tol), (li, an, f32, fd)


def test_bptt_full_config_runs_and_learns():
    """The full differentiation config (784-512-512-10, batch 128, T = 32, checkpoint 8): SGD steps
    on one batch lower the cross-entropy of the output spike counts."""
    from knp_gb300 import bptt

    x, labels = bptt.make_batch(T=32, B=128, seed=7)
    model = bptt.SpikingMLP(sizes=(784, 512, 512, 10), checkpoint=8, seed=3)
    opt = torch.optim.SGD(model.parameters(), lr=1e-4)
    losses = []
    for _ in range(10):
        opt.zero_grad(set_to_none=True)
        loss = bptt.loss_fn(model(x), labels)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    assert all(torch.isfinite(torch.tensor(losses)))
    assert losses[-1] < losses[0], losses


def test_graphed_train_step_matches_eager_steps():
    """GraphedTrainStep (the iteration captured once as a CUDA graph) takes the same SGD steps as the
    eager loop: after 3 warm-up + 4 replayed iterations the weights and the loss equal those of 7 eager
    iterations bit for bit (every kernel of the iteration is deterministic, split-K GEMMs included)."""
    from knp_gb300 import bptt

    x, labels = bptt.make_batch(T=16, B=64, seed=5)
    eager = bptt.SpikingMLP(sizes=(784, 256, 10), checkpoint=8, seed=4)
    graphed = bptt.SpikingMLP(sizes=(784, 256, 10), checkpoint=8, seed=4)
    opt_e = torch.optim.SGD(eager.parameters(), lr=1e-3)
    opt_g = torch.optim.SGD(graphed.parameters(), lr=1e-3)
    for _ in range(7):
        opt_e.zero_grad(set_to_none=True)
        loss_e = bptt.loss_fn(eager(x), labels)
        loss_e.backward()
        opt_e.step()
    step = bptt.GraphedTrainStep(graphed, opt_g, x, labels, warmup=3)
    for _ in range(4):
        loss_g = step()
    torch.cuda.synchronize()
    bptt.check_gemm_errors()
    assert torch.equal(loss_g, loss_e)
    for a, b in zip(eager.weights, graphed.weights):
        assert torch.equal(a, b)


def test_fused_operands_equal_the_torch_composition(monkeypatch):
    """knp_gb300_bf16_operand builds the same GEMM operands as the torch composition (cast, hi/lo
    split, transposes, concatenation and padding along K): loss and every weight gradient are equal
    bit for bit, with a layer width that needs padding (10 outputs)."""
    from knp_gb300 import bptt

    x, labels = bptt.make_batch(T=12, B=41, n_in=200, seed=8)  # T B = 492: K padded to 496
    grads = []
    for fused in (True, False):
        monkeypatch.setattr(bptt, "FUSED_OPERANDS", fused)
        model = bptt.SpikingMLP(sizes=(200, 136, 10), checkpoint=4, seed=6)
        loss = bptt.loss_fn(model(x), labels)
        loss.backward()
        torch.cuda.synchronize()
        grads.append((loss.detach().clone(), [w.grad.clone() for w in model.weights]))
    bptt.check_gemm_errors()
    assert torch.equal(grads[0][0], grads[1][0])
    for a, b in zip(grads[0][1], grads[1][1]):
        assert torch.equal(a, b)
