"""PrideDiff's data-consistency block (model/pridediff.py:9-68) on this
library: pridediff_gb300.fidelity.FidelityModule with PrideDiff's FBP adjoint
and with the exact adjoint, its autograd pairing, and graph capture."""
import numpy as np
import pytest
import torch

from conftest import rel_l2


def test_default_geometry_is_pridediffs():
    from pridediff_gb300.fidelity import FidelityModule
    m = FidelityModule()
    o = m.proj.options.detach().numpy().astype(np.float64)
    # [W, H, D, sx, sy, det (rad), SID, SDD, px, py, bin]: arc det pitch 1.2858 / 490.6
    assert list(o[:3]) == [512, 512, 768] and m.proj.scan_type == "arc"
    assert np.allclose(o[3:8], [0.7433, 0.7433, 1.2858 / 490.6, 595.0, 490.6], rtol=1e-7)
    assert m.views.numel() == 720 and abs(float(m.views[1]) - 2 * np.pi / 720) < 1e-7
    with pytest.raises(ValueError):
        FidelityModule(adjoint="other")


def _small(adjoint):
    from pridediff_gb300.fidelity import FidelityModule
    from pridediff_gb300.projector import projector2d
    proj = projector2d(64, 96, 1.4, 1.2858, 595.0, 1085.6, scan_type="arc")
    views = torch.arange(90) * torch.pi * 2 / 90
    m = FidelityModule(proj, views, adjoint).cuda()
    with torch.no_grad():
        m.weight.fill_(0.3)
    g = torch.Generator().manual_seed(4)
    x = torch.rand(2, 1, 64, 64, generator=g).cuda()
    y = torch.rand(2, 1, 90, 96, generator=g).cuda()
    return m, x, y


@pytest.mark.gpu
@pytest.mark.parametrize("adjoint", ["fbp", "exact"])
def test_gpu_fidelity_step_is_the_composition(adjoint):
    m, x, y = _small(adjoint)
    with torch.no_grad():
        out = m(x, y, None)
        r = m.proj.projection(x, m.views) - y
        at = m.proj.filtered_backprojection(r, m.views) if adjoint == "fbp" else m.proj.projection_t(r, m.views)
        ref = x - 0.3 * at
    assert torch.equal(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("adjoint", ["fbp", "exact"])
def test_gpu_projection_backward_uses_the_modules_adjoint(adjoint):
    from pridediff_gb300.fidelity import _Prj
    m, x, y = _small(adjoint)
    x = x.clone().requires_grad_(True)
    (_Prj.apply(x, m) * y).sum().backward()
    ref = m.adjoint_op(y)
    assert rel_l2(x.grad.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    if adjoint == "exact":   # the true transpose: <A x, y> = <x, A^T y>
        with torch.no_grad():
            lhs = float((m.proj.projection(x, m.views).double() * y.double()).sum())
            rhs = float((x.double() * ref.double()).sum())
        assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


@pytest.mark.gpu
def test_gpu_fidelity_graph_replays_the_eager_steps():
    from pridediff_gb300.fidelity import fidelity_graph
    m, x, y = _small("fbp")
    xe = x.clone()
    with torch.no_grad():
        for _ in range(3):
            xe = m(xe, y)
    xg = x.clone()
    graph = fidelity_graph(m, xg, y, steps=3)
    graph.replay()
    torch.cuda.synchronize()
    assert rel_l2(xg.cpu().numpy(), xe.cpu().numpy()) <= 1e-6


class _TinyDenoiser(torch.nn.Module):
    """A small stock-PyTorch network standing in for PrideDiff's UNet."""

    def __init__(self):
        super().__init__()
        self.c1 = torch.nn.Conv2d(1, 8, 3, padding=1)
        self.c2 = torch.nn.Conv2d(8, 1, 3, padding=1)
        self.t = torch.nn.Embedding(16, 8)

    def forward(self, x, t):
        h = torch.relu(self.c1(x) + self.t(t)[:, :, None, None])
        return x + 0.1 * self.c2(h)


class _LearnBlock(torch.nn.Module):
    """PrideDiff's IterBlock (model/pridediff.py:137-151): relu(DC(x) + cnn(x))."""

    def __init__(self, dc):
        super().__init__()
        self.dc = dc
        self.cnn = torch.nn.Conv2d(1, 1, 3, padding=1)

    def forward(self, x, sino, t):
        return torch.relu(self.dc(x, sino, t) + 0.05 * self.cnn(x))


@pytest.mark.gpu
def test_gpu_sampling_loop_with_graph_captured_dc_matches_eager():
    """GaussianDiffusion.sample's loop (model/pridediff.py:256-298) with a
    stock-PyTorch denoiser, its learn block's data-consistency step replayed
    from a CUDA graph at every step, equals the same loop run eagerly."""
    from pridediff_gb300.fidelity import GraphedFidelity, sample
    m, x, y = _small("exact")
    torch.manual_seed(0)
    den = _TinyDenoiser().cuda().eval()
    steps = 10
    alphas = torch.clip(1 - torch.linspace(0, steps, steps) / steps, 0, 0.999).cuda()
    eager = _LearnBlock(m).cuda().eval()
    with torch.no_grad():
        sino = m.proj.projection(x, m.views)
    g = GraphedFidelity(m, x, sino)
    g.set_sino(sino)
    graphed = _LearnBlock(g).cuda().eval()
    graphed.cnn.load_state_dict(eager.cnn.state_dict())
    _, d_e, out_e = sample(den, eager, x, sino, alphas)
    _, d_g, out_g = sample(den, graphed, x, sino, alphas)
    torch.cuda.synchronize()
    assert rel_l2(d_g.cpu().numpy(), d_e.cpu().numpy()) <= 1e-6
    assert rel_l2(out_g.cpu().numpy(), out_e.cpu().numpy()) <= 1e-6
    # the graph replays the module's current weight: loading another one in place needs no recapture
    with torch.no_grad():
        m.weight.fill_(0.1)
    _, _, out_e2 = sample(den, eager, x, sino, alphas)
    _, _, out_g2 = sample(den, graphed, x, sino, alphas)
    assert rel_l2(out_g2.cpu().numpy(), out_e2.cpu().numpy()) <= 1e-6
    assert rel_l2(out_g2.cpu().numpy(), out_g.cpu().numpy()) > 1e-4
