"""The tensor-memory convolution (tcgen05 + TMA) against the warp-MMA kernel
and the FP64 oracle, over the channel counts and box shapes the U-Net uses."""
import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import unet_oracle as U  # noqa: E402

CASES = [
    # (batch, nz, ny, nx, cin, cout)
    (1, 32, 32, 32, 16, 32),    # first layer: 32-byte swizzle
    (2, 16, 16, 16, 32, 64),    # 64-byte swizzle
    (1, 16, 16, 16, 64, 128),   # 128-byte swizzle
    (2, 8, 8, 8, 128, 256),     # box spans z
    (4, 4, 4, 4, 256, 128),     # box spans the batch
    (1, 8, 16, 32, 256, 256),   # non-cubic
    (1, 16, 16, 16, 64, 32),
    (1, 8, 8, 8, 256, 256),     # 4 tiles: reduction split into 19 tap ranges
]


def run(case, path, relu, seed=0):
    import torch
    from doma_gb300 import abi
    b, z, y, x, cin, cout = case
    rng = np.random.default_rng(seed)
    xs = rng.normal(0, 1, (b, z, y, x, cin)).astype(np.float32)
    ws = rng.normal(0, 1 / np.sqrt(27 * cin), (27, cout, cin)).astype(np.float32)
    bias = rng.normal(0, 0.1, cout).astype(np.float32)
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(xs).to(dev).to(torch.bfloat16).contiguous()
    wd = torch.from_numpy(ws).to(dev).to(torch.bfloat16).contiguous()
    bd = torch.from_numpy(bias).to(dev)
    yd = torch.full((b, z, y, x, cout), float("nan"), device=dev).to(torch.bfloat16)
    lib = abi.load_library()
    st = lib.doma_conv3_forward(ctypes.c_void_p(xd.data_ptr()), b, z, y, x, cin,
                                ctypes.c_void_p(wd.data_ptr()),
                                ctypes.cast(ctypes.c_void_p(bd.data_ptr()), ctypes.c_void_p),
                                cout, int(relu), ctypes.c_void_p(yd.data_ptr()), path, None)
    abi.check(st, "doma_conv3_forward", lib)
    torch.cuda.synchronize()
    flag = ctypes.c_int(-1)
    abi.check(lib.doma_conv_wait_error(ctypes.byref(flag)), "doma_conv_wait_error", lib)
    assert flag.value == 0
    got = yd.float().cpu().numpy().astype(np.float64)
    want = U.conv(U.round_bf16(xs), U.round_bf16(ws), bias.astype(np.float64))
    if relu:
        want = np.maximum(want, 0.0)
    return got, want


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_tensor_memory_conv_matches_the_oracle(case):
    from doma_gb300 import abi
    got, want = run(case, abi.DOMA_CONV_TENSOR_MEMORY, relu=True)
    assert np.all(np.isfinite(got))
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 5e-3, err


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(2, 16, 16, 16, 64, 64), (1, 16, 16, 16, 128, 128)])
def test_tensor_memory_and_mma_kernels_agree(case):
    # the second shape has 32 tiles, so the tensor-memory kernel splits its reduction
    from doma_gb300 import abi
    a, want = run(case, abi.DOMA_CONV_TENSOR_MEMORY, relu=False, seed=3)
    b, _ = run(case, abi.DOMA_CONV_MMA, relu=False, seed=3)
    assert np.linalg.norm(a - b) / np.linalg.norm(want) < 5e-3
    assert np.linalg.norm(b - want) / np.linalg.norm(want) < 5e-3


@pytest.mark.gpu
def test_split_reduction_is_deterministic():
    from doma_gb300 import abi
    case = (1, 8, 8, 8, 256, 128)
    a, _ = run(case, abi.DOMA_CONV_TENSOR_MEMORY, relu=True, seed=7)
    b, _ = run(case, abi.DOMA_CONV_TENSOR_MEMORY, relu=True, seed=7)
    assert np.array_equal(a, b)


def test_conv_path_constants_are_exported():
    from doma_gb300 import abi
    assert (abi.DOMA_CONV_AUTO, abi.DOMA_CONV_MMA, abi.DOMA_CONV_TENSOR_MEMORY) == (0, 1, 2)


WGRAD_CASES = CASES + [
    (1, 64, 64, 64, 32, 32),    # the 64^3 level: 4 taps of 32 channels per MMA
    (1, 8, 8, 8, 256, 256),     # two 128-channel blocks, one tap per MMA
]


def run_wgrad(case, path, seed=0):
    import torch
    from doma_gb300 import abi
    b, z, y, x, cin, cout = case
    rng = np.random.default_rng(seed)
    xs = rng.normal(0, 1, (b, z, y, x, cin)).astype(np.float32)
    gs = rng.normal(0, 1, (b, z, y, x, cout)).astype(np.float32)
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(xs).to(dev).to(torch.bfloat16).contiguous()
    gd = torch.from_numpy(gs).to(dev).to(torch.bfloat16).contiguous()
    dw = torch.full((27, cout, cin), float("nan"), device=dev)
    lib = abi.load_library()
    st = lib.doma_conv3_wgrad(ctypes.c_void_p(xd.data_ptr()), b, z, y, x, cin,
                              ctypes.c_void_p(gd.data_ptr()), cout,
                              ctypes.c_void_p(dw.data_ptr()), path, None)
    abi.check(st, "doma_conv3_wgrad", lib)
    torch.cuda.synchronize()
    flag = ctypes.c_int(-1)
    abi.check(lib.doma_conv_wait_error(ctypes.byref(flag)), "doma_conv_wait_error", lib)
    assert flag.value == 0
    return dw.cpu().numpy().astype(np.float64), xs, gs


@pytest.mark.gpu
@pytest.mark.parametrize("case", WGRAD_CASES)
def test_tensor_memory_wgrad_matches_the_oracle(case):
    """The tensor-core weight gradient (taps stacked along the MMA rows,
    MN-major operands straight from TMA) against the FP64 oracle on the same
    bf16 inputs, and against the warp-MMA kernel."""
    from doma_gb300 import abi
    got, xs, gs = run_wgrad(case, abi.DOMA_CONV_TENSOR_MEMORY, seed=5)
    want = U.conv_wgrad(U.round_bf16(xs), U.round_bf16(gs))
    assert np.all(np.isfinite(got))
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 1e-4, err
    mma, _, _ = run_wgrad(case, abi.DOMA_CONV_MMA, seed=5)
    assert np.linalg.norm(mma - want) / np.linalg.norm(want) < 1e-4


@pytest.mark.gpu
def test_tensor_memory_wgrad_is_deterministic():
    from doma_gb300 import abi
    case = (1, 16, 16, 16, 64, 64)
    a, _, _ = run_wgrad(case, abi.DOMA_CONV_TENSOR_MEMORY, seed=9)
    b, _, _ = run_wgrad(case, abi.DOMA_CONV_TENSOR_MEMORY, seed=9)
    assert np.array_equal(a, b)


@pytest.mark.gpu
def test_halo_kernel_on_every_shape_it_supports():
    """The halo-tile kernel runs by default for 16-channel inputs only; with
    DOMA_CONV_HALO=1 (read once per process, hence the child process) it takes
    every shape it supports, 32-channel inputs included, and must pass the
    same oracle comparisons."""
    import os
    import subprocess
    env = dict(os.environ, DOMA_CONV_HALO="1")
    r = subprocess.run([sys.executable, "-m", "pytest", __file__, "-q", "-m", "gpu",
                        "-p", "no:cacheprovider", "-k", "tensor_memory_conv_matches_the_oracle"],
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
