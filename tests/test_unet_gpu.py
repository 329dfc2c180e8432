"""The warm-start U-Net on the GPU against the PyTorch CPU FP32 oracle
(oracle/unet_ref.py) that rounds to BF16 where the GPU stores BF16: forward
output, loss gradients and one Adam step.  Accumulation order differs
(tensor-core tiles, FP32 atomics), so agreement is to BF16 rounding:
relative L2 below 2e-2 for outputs, 5e-2 per parameter block for
gradients."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SH = (16, 12, 8)
H = 1.0 / 16


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def inputs(seed=0, sh=SH):
    rng = np.random.default_rng(seed)
    n = sh[0] * sh[1] * sh[2]
    k, j, i = np.meshgrid(np.arange(sh[2]), np.arange(sh[1]), np.arange(sh[0]), indexing="ij")
    b = (np.sin(2 * np.pi * i / sh[0]) * np.cos(2 * np.pi * j / sh[1]) + 0.3 * rng.standard_normal(i.shape))
    b = b.astype(np.float32).ravel()
    mask = (rng.random(n) < 0.1).astype(np.uint8)
    pp = rng.standard_normal(n).astype(np.float32) * 0.01
    target = rng.standard_normal(n).astype(np.float32) * 0.02
    return b, mask, pp, target


def fields(b, mask, pp, target, sh=SH):
    from tsl_array_n_gb300.tsl_array_n import Field
    return (Field("float", sh).from_array(b), Field("uint8", sh).from_array(mask),
            Field("float", sh).from_array(pp), Field("float", sh).from_array(target))


def test_param_count(gpu):
    from oracle import unet_ref
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=3)
    assert net.param_count == unet_ref.param_count()
    assert 300_000 < net.param_count < 400_000


def test_forward_matches_torch(gpu):
    from oracle import unet_ref
    from tsl_array_n_gb300.tsl_array_n import Field
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=5)
    b, mask, pp, target = inputs(1)
    fb, fm, fp, _ = fields(b, mask, pp, target)
    out = Field("float", SH)
    net.forward(SH, H, fb, fm, fp, out)
    ref = unet_ref.predict(net.params, b, mask, pp, H, SH)
    assert rel(out.to_array(), ref) < 2e-2
    # without a previous pressure the second scale comes from b
    net.forward(SH, H, fb, fm, None, out)
    ref = unet_ref.predict(net.params, b, mask, None, H, SH)
    assert rel(out.to_array(), ref) < 2e-2


@pytest.mark.parametrize("sh", [(40, 36, 64), (24, 20, 32)])
def test_forward_matches_torch_long_columns(gpu, sh):
    """Volumes whose convolutions split each tile column into several z
    ranges, with partial tiles at the y edge (36 and 20 rows against tiles
    of 16)."""
    from oracle import unet_ref
    from tsl_array_n_gb300.tsl_array_n import Field
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=13)
    b, mask, pp, target = inputs(5, sh)
    fb, fm, fp, _ = fields(b, mask, pp, target, sh)
    out = Field("float", sh)
    net.forward(sh, 1.0 / sh[0], fb, fm, fp, out)
    ref = unet_ref.predict(net.params, b, mask, pp, 1.0 / sh[0], sh)
    assert rel(out.to_array(), ref) < 2e-2


def test_gradients_match_torch_long_columns(gpu):
    from oracle import unet_ref
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    sh = (24, 20, 32)
    net = UNetWarmStart(seed=17)
    b, mask, pp, target = inputs(6, sh)
    loss = net.loss_backward(sh, 1.0 / sh[0], *fields(b, mask, pp, target, sh))
    ref_loss, ref_g = unet_ref.loss_and_grads(net.params, b, mask, pp, target, 1.0 / sh[0], sh)
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    g = net.grads
    off = 0
    for ci, co in unet_ref.SPEC:
        nw = 27 * ci * co
        assert rel(g[off:off + nw], ref_g[off:off + nw]) < 5e-2, (ci, co)
        off += nw + co


def test_gradients_match_torch(gpu):
    from oracle import unet_ref
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=7)
    b, mask, pp, target = inputs(2)
    loss = net.loss_backward(SH, H, *fields(b, mask, pp, target))
    ref_loss, ref_g = unet_ref.loss_and_grads(net.params, b, mask, pp, target, H, SH)
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    g = net.grads
    off = 0
    for ci, co in unet_ref.SPEC:
        nw = 27 * ci * co
        assert rel(g[off:off + nw], ref_g[off:off + nw]) < 5e-2, (ci, co)
        assert rel(g[off + nw:off + nw + co], ref_g[off + nw:off + nw + co]) < 5e-2, (ci, co, "bias")
        off += nw + co
    assert rel(g[off:], ref_g[off:]) < 2e-2


def test_adam_step_matches_reference(gpu):
    from oracle import unet_ref
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=9)
    b, mask, pp, target = inputs(3)
    p0 = net.params
    net.loss_backward(SH, H, *fields(b, mask, pp, target))
    g = net.grads
    net.adam_step(lr=1e-3)
    want, _, _ = unet_ref.adam(p0.astype(np.float64), g.astype(np.float64), 0.0, 0.0, 1, 1e-3)
    np.testing.assert_allclose(net.params, want, rtol=1e-5, atol=1e-7)


def test_training_lowers_the_loss(gpu):
    from tsl_array_n_gb300.warmstart import UNetWarmStart
    net = UNetWarmStart(seed=11)
    b, mask, pp, target = inputs(4)
    fs = fields(b, mask, pp, target)
    first = net.train_step(SH, H, *fs, lr=3e-3)
    for _ in range(40):
        last = net.train_step(SH, H, *fs, lr=3e-3)
    assert last < 0.5 * first
