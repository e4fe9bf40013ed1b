"""The radiance-cache network on the tensor cores against its FP64 numpy
definition (oracle/mlp.py): inference, gradients, and that training on the
GPU lowers the loss.  Tolerances: outputs agree to 1e-3 relative (FP32
accumulation of FP16 products); gradients to 2e-2 in relative norm per layer
(FP16 rounding of intermediate gradients amplified through five layers)."""
import ctypes

import numpy as np
import pytest

from oracle import mlp as ref

pytestmark = pytest.mark.gpu


@pytest.fixture()
def net(gpu_lib):
    from craystal_gb300._lib import CrMlpConfig, check, load
    cfg = CrMlpConfig(1e-2, 0.9, 0.99, 1e-8, 7)
    h = ctypes.c_void_p()
    check(load().cr_mlp_create(ctypes.byref(cfg), ctypes.byref(h)))
    yield h
    load().cr_mlp_destroy(h)


def _params(h):
    from craystal_gb300._lib import check, load, ptr
    p = np.zeros(load().cr_mlp_param_count(), np.float32)
    check(load().cr_mlp_get_params(h, ptr(p)))
    return p


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 7)).astype(np.float32)
    t = (0.5 + 0.4 * np.sin(6 * x[:, :3]) * np.cos(3 * x[:, 3:6])).astype(np.float32)
    return x, t


def test_param_count_and_layout(gpu_lib):
    from craystal_gb300._lib import load
    assert load().cr_mlp_param_count() == ref.N_PARAMS == 27840


def test_inference_matches_fp64(net):
    from craystal_gb300._lib import check, load, ptr
    x, _ = _inputs(3000, 1)
    out = np.zeros((len(x), 3), np.float32)
    check(load().cr_mlp_infer(net, ptr(x), len(x), ptr(out)))
    y, _ = ref.forward(_params(net), x)
    np.testing.assert_allclose(out, y, rtol=1e-3, atol=1e-3 * np.abs(y).max())


@pytest.mark.parametrize("n", [1, 127, 128, 129, 383, 385, 70001, 233549])
def test_inference_ragged_batches(net, n):
    """Tensor-core inference over partial tiles (128 queries per tile, three
    tiles per CTA in flight), over grids of one CTA up to one per SM, and
    with several tiles per warpgroup (233,549 queries: four or more each)."""
    from craystal_gb300._lib import check, load, ptr
    x, _ = _inputs(n, 10 + n)
    out = np.full((n, 3), np.nan, np.float32)
    check(load().cr_mlp_infer(net, ptr(x), n, ptr(out)))
    y, _ = ref.forward(_params(net), x)
    assert np.isfinite(out).all()
    np.testing.assert_allclose(out, y, rtol=1e-3, atol=1e-3 * np.abs(y).max())


def test_gradients_match_fp64(net):
    from craystal_gb300._lib import check, load, ptr
    x, t = _inputs(4096, 2)
    g = np.zeros(load().cr_mlp_param_count(), np.float32)
    loss = ctypes.c_float()
    check(load().cr_mlp_gradients(net, ptr(x), ptr(t), len(x), ptr(g), ctypes.byref(loss)))
    lref, gref = ref.loss_and_grads(_params(net), x, t)
    assert abs(loss.value - lref) <= 1e-3 * lref
    o = 0
    for k, n in ref.SHAPES:
        a, b = g[o:o + k * n], gref[o:o + k * n]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), (k, n)
        o += k * n


@pytest.mark.parametrize("n", [1, 100, 128, 129, 20000, 70001])
def test_gradients_ragged_batches(net, n):
    """The training kernel over partial tiles (128 records per tile) and over
    grids of one CTA up to one per SM (each CTA sums its tiles' weight
    gradients in TMEM and contributes one partial): per-layer gradients
    against the FP64 definition, and the loss."""
    from craystal_gb300._lib import check, load, ptr
    x, t = _inputs(n, 20 + n)
    g = np.zeros(load().cr_mlp_param_count(), np.float32)
    loss = ctypes.c_float()
    check(load().cr_mlp_gradients(net, ptr(x), ptr(t), n, ptr(g), ctypes.byref(loss)))
    lref, gref = ref.loss_and_grads(_params(net), x, t)
    assert abs(loss.value - lref) <= 1e-3 * lref
    assert np.isfinite(g).all()
    o = 0
    for k, m in ref.SHAPES:
        a, b = g[o:o + k * m], gref[o:o + k * m]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), (n, k, m)
        o += k * m


def test_training_reduces_loss(net):
    from craystal_gb300._lib import check, load, ptr
    x, t = _inputs(1 << 14, 3)
    losses = []
    for _ in range(300):
        loss = ctypes.c_float()
        check(load().cr_mlp_train_step(net, ptr(x), ptr(t), len(x), ctypes.byref(loss)))
        losses.append(loss.value)
    assert losses[-1] < 0.1 * losses[0], (losses[0], losses[-1])


def test_adam_step_matches_fp64(net):
    """One GPU Adam step equals the FP64 update computed from the GPU's own
    gradient (isolates the optimiser from gradient rounding)."""
    from craystal_gb300._lib import check, load, ptr
    x, t = _inputs(2048, 4)
    p0 = _params(net).astype(np.float64)
    g = np.zeros(load().cr_mlp_param_count(), np.float32)
    check(load().cr_mlp_gradients(net, ptr(x), ptr(t), len(x), ptr(g), None))
    check(load().cr_mlp_train_step(net, ptr(x), ptr(t), len(x), None))
    p1 = _params(net)
    expect, _, _ = ref.adam_step(p0, 0.0, 0.0, g.astype(np.float64), 1)
    # the first Adam step moves each weight by lr * g / (|g| + eps); compare
    # where |g| is well above the float rounding noise of the two gradient passes
    m = np.abs(g) > 1e-6
    assert m.mean() > 0.5
    np.testing.assert_allclose(p1[m], expect[m], rtol=1e-5, atol=1e-6)


def test_inference_unaligned_device_inputs(net):
    """Device inputs that start off a 16-byte boundary (each query's 7 floats
    are read as plain 4-byte loads) give the host form's outputs."""
    import torch
    from craystal_gb300._lib import check, load, ptr
    x, _ = _inputs(50001, 12)
    ref_out = np.zeros((len(x), 3), np.float32)
    check(load().cr_mlp_infer(net, ptr(x), len(x), ptr(ref_out)))
    buf = torch.zeros(len(x) * 7 + 1, dtype=torch.float32, device="cuda")
    buf[1:] = torch.from_numpy(x.reshape(-1)).cuda()
    assert (buf.data_ptr() + 4) % 16 != 0
    dout = torch.empty((len(x), 3), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    check(load().cr_mlp_infer_device(net, buf.data_ptr() + 4, len(x), dout.data_ptr(), s.cuda_stream))
    s.synchronize()
    assert np.array_equal(dout.cpu().numpy(), ref_out)


def test_device_forms_match_host_forms(gpu_lib):
    """cr_mlp_infer_device / cr_mlp_train_step_device (device buffers, the
    calls the cached integrator makes) give what the host-buffer forms give."""
    import torch
    from craystal_gb300._lib import CrMlpConfig, check, load, ptr
    lib = load()
    nets = []
    for _ in range(2):
        h = ctypes.c_void_p()
        check(lib.cr_mlp_create(ctypes.byref(CrMlpConfig(1e-2, 0.9, 0.99, 1e-8, 11)), ctypes.byref(h)))
        nets.append(h)
    try:
        x, t = _inputs(5000, 5)
        out_h = np.zeros((len(x), 3), np.float32)
        check(lib.cr_mlp_infer(nets[0], ptr(x), len(x), ptr(out_h)))
        dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        dout = torch.empty((len(x), 3), dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream()
        check(lib.cr_mlp_infer_device(nets[1], dx.data_ptr(), len(x), dout.data_ptr(), s.cuda_stream))
        assert np.array_equal(dout.cpu().numpy(), out_h)
        g = np.zeros(lib.cr_mlp_param_count(), np.float32)
        check(lib.cr_mlp_gradients(nets[0], ptr(x), ptr(t), len(x), ptr(g), None))
        check(lib.cr_mlp_train_step(nets[0], ptr(x), ptr(t), len(x), None))
        check(lib.cr_mlp_train_step_device(nets[1], dx.data_ptr(), dt.data_ptr(), len(x), s.cuda_stream))
        torch.cuda.synchronize()
        p0, p1 = _params(nets[0]), _params(nets[1])
        # the CTAs' gradient partials are summed in a fixed order, so the two
        # forms take the same step bit for bit
        assert np.array_equal(p1.view(np.uint32), p0.view(np.uint32))
        assert (np.abs(g) > 1e-6).mean() > 0.5
        # a second device step keeps training: the loss goes down
        for _ in range(50):
            check(lib.cr_mlp_train_step_device(nets[1], dx.data_ptr(), dt.data_ptr(), len(x), s.cuda_stream))
        torch.cuda.synchronize()
        l0, _ = ref.loss_and_grads(p0, x, t)
        l1, _ = ref.loss_and_grads(_params(nets[1]), x, t)
        assert l1 < l0
    finally:
        for h in nets:
            lib.cr_mlp_destroy(h)
