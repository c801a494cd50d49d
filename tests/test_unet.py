"""The learned accelerator's network: the CPU oracle's calculus (finite
differences), and the GPU kernels' forward pass and gradients against the
oracle with BF16 rounding at the same points."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import unet_oracle as U  # noqa: E402


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    offs, head, n = U.layout()
    flat = np.zeros(n, dtype=np.float32)
    for (cin, cout, relu), (wo, bo) in zip(U.LAYERS, offs):
        fan = 27 * (3 if cin == U.IN_CH else cin)
        w = rng.normal(0, np.sqrt((2.0 if relu else 1.0) / fan), (27, cout, cin)) * scale
        if cin == U.IN_CH:
            w[:, :, 3:] = 0.0
        flat[wo:wo + w.size] = w.reshape(-1)
        flat[bo:bo + cout] = rng.normal(0, 0.05, cout)
    flat[head[0]:head[0] + 32] = rng.normal(0, 0.3, 32)
    flat[head[1]] = 0.1
    return flat


def random_input(seed, shape):
    rng = np.random.default_rng(seed)
    x = np.zeros(shape + (U.IN_CH,), dtype=np.float32)
    x[..., :3] = rng.normal(0, 1, shape + (3,))
    t = rng.normal(0, 1, shape).astype(np.float32)
    return x, t


def test_layout_matches_the_documented_parameter_count():
    _, _, n = U.layout()
    assert n == 5_268_385


def test_oracle_gradient_matches_finite_differences():
    flat = random_params(1).astype(np.float64)
    x, t = random_input(2, (1, 8, 8, 8))
    _, g, _ = U.loss_and_grads(flat, x, t, bf16=False)
    rng = np.random.default_rng(3)
    for k in range(3):
        v = rng.normal(0, 1, flat.size)
        v[np.abs(flat) == 0] = 0.0  # keep the padded input channels out
        fd = U.finite_difference(flat, x, t, v, eps=1e-8)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (k, fd, an)


def test_oracle_bf16_rounding_is_round_to_nearest_even():
    a = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e-3], dtype=np.float32)
    r = U.round_bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert r[3] == -2.5


def _gpu_case(shape, seed):
    import torch
    from doma_gb300.learned.net import UNet
    flat = random_params(seed)
    x, t = random_input(seed + 1, shape)
    net = UNet(seed=0)
    net.set_params(flat)
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(x).to(dev).to(torch.bfloat16).contiguous()
    td = torch.from_numpy(t).to(dev).contiguous()
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    net.forward(xd, out)
    torch.cuda.synchronize()
    got_out = out.cpu().numpy()
    net.backward(xd, td)
    got_loss = net.loss()
    got_g = net.grads()
    net.close()
    loss, g, want_out = U.loss_and_grads(flat, x, t, bf16=True)
    return got_out, got_loss, got_g, want_out, loss, g


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(2, 8, 8, 8), (1, 8, 16, 24)])
def test_gpu_forward_and_gradients_match_the_oracle(shape):
    got_out, got_loss, got_g, want_out, loss, g = _gpu_case(shape, seed=5)
    assert rel(got_out, want_out) < 1e-2
    assert abs(got_loss - loss) <= 2e-2 * loss
    offs, head, _ = U.layout()
    for k, ((cin, cout, _), (wo, bo)) in enumerate(zip(U.LAYERS, offs)):
        n = 27 * cin * cout
        assert rel(got_g[wo:wo + n], g[wo:wo + n]) < 3e-2, ("weights", k)
        assert rel(got_g[bo:bo + cout], g[bo:bo + cout]) < 3e-2, ("bias", k)
    assert rel(got_g[head[0]:head[0] + 33], g[head[0]:head[0] + 33]) < 1e-2


@pytest.mark.gpu
def test_gpu_adam_training_reduces_the_loss():
    import torch
    from doma_gb300.learned.net import UNet
    x, t = random_input(11, (4, 16, 16, 16))
    # a smooth target the network can fit: a blurred copy of input channel 0
    t = x[..., 0].copy()
    for ax in (1, 2, 3):
        t = (np.roll(t, 1, ax) + t + np.roll(t, -1, ax)) / 3.0
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(x).to(dev).to(torch.bfloat16).contiguous()
    td = torch.from_numpy(t.astype(np.float32)).to(dev).contiguous()
    net = UNet(seed=3)
    net.backward(xd, td)
    first = net.loss()
    for _ in range(60):
        net.backward(xd, td)
        net.adam(1e-3)
    net.backward(xd, td)
    last = net.loss()
    net.close()
    assert last < 0.5 * first, (first, last)


@pytest.mark.gpu
def test_weighted_loss_scales_each_sample():
    """doma_unet_backward_weighted: unit weights give the unweighted gradient,
    a uniform weight of 2 doubles every gradient exactly (a power of two), and
    a zero weight removes a sample: with weights (2, 0) the gradients do not
    depend on the second sample at all (swapping it for another one leaves
    every bit unchanged)."""
    import torch

    from doma_gb300.learned.net import UNet
    torch.cuda.set_device(0)
    flat = random_params(11)
    x, t = random_input(12, (2, 16, 16, 16))
    x2, t2 = random_input(13, (2, 16, 16, 16))
    x2[0], t2[0] = x[0], t[0]
    xd = torch.from_numpy(x).cuda().to(torch.bfloat16).contiguous()
    td = torch.from_numpy(t).cuda().contiguous()
    xd2 = torch.from_numpy(x2).cuda().to(torch.bfloat16).contiguous()
    td2 = torch.from_numpy(t2).cuda().contiguous()
    with UNet(seed=1) as net:
        net.set_params(flat)
        net.backward(xd, td)
        g1 = net.grads().copy()
        l1 = net.loss()
        net.backward(xd, td, torch.ones(2, device="cuda"))
        assert np.array_equal(net.grads(), g1)
        net.backward(xd, td, torch.full((2,), 2.0, device="cuda"))
        assert np.array_equal(net.grads(), 2.0 * g1)
        assert net.loss() == pytest.approx(2.0 * l1, rel=1e-12)
        w = torch.tensor([2.0, 0.0], device="cuda")
        net.backward(xd, td, w)
        ga = net.grads().copy()
        net.backward(xd2, td2, w)
        gb = net.grads().copy()
    assert np.abs(ga).max() > 0
    assert np.array_equal(ga, gb)
