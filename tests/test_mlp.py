"""The LSMC continuation network: its CPU gradients against finite differences, the
tensor-core training kernel's gradients against the CPU oracle, and LSMC pricing with
the trained network judged by the Heston ADI price."""
import ctypes as C
import math

import numpy as np
import pytest

from kiyosi_gb300 import abi
from kiyosi_gb300.market import HestonParameters, PricingContext
from oracle import loader

from helpers import gpu_lsmc, lsmc_settings

GROUPS = {"W1": (0, 192), "b1": (192, 256), "W2": (256, 4352), "b2": (4352, 4416),
          "w3": (4416, 4480), "b3": (4480, 4481)}


def _params(seed=3):
    rng = np.random.default_rng(seed)
    p = np.zeros(abi.MLP_PARAMS, np.float32)
    p[0:192] = rng.uniform(-1.4, 1.4, 192)
    p[192:256] = rng.uniform(-0.1, 0.1, 64)
    p[256:4352] = rng.uniform(-0.3, 0.3, 4096)
    p[4352:4416] = rng.uniform(-0.1, 0.1, 64)
    p[4416:4480] = rng.uniform(-0.3, 0.3, 64)
    p[4480] = 0.05
    return p


def _samples(n, seed=5):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 4)).astype(np.float32)
    x[:, 2] = rng.uniform(0.0, 1.0, n)
    x[:, 3] = np.abs(x[:, 3]) * 0.1
    return x


def test_oracle_gradients_match_finite_differences():
    p, x = _params(), _samples(300)
    _, g = loader.mlp_gradients(p, x, bf16_operands=False)
    for idx in (0, 100, 191, 300, 1000, 4000, 4351, 4415, 4420, 4479, 4480):
        h = 1e-6 * max(1.0, abs(float(p[idx])))
        q_plus, q_minus = p.copy(), p.copy()
        q_plus[idx] = np.float32(float(p[idx]) + h)
        q_minus[idx] = np.float32(float(p[idx]) - h)
        lp, _ = loader.mlp_gradients(q_plus, x, bf16_operands=False)
        lm, _ = loader.mlp_gradients(q_minus, x, bf16_operands=False)
        fd = (lp - lm) / (float(q_plus[idx]) - float(q_minus[idx]))
        assert abs(g[idx] - fd) <= 1e-6 * max(1.0, abs(fd)), (idx, g[idx], fd)


@pytest.mark.gpu
@pytest.mark.parametrize("count", [128, 1000, 8192])
def test_tensor_core_gradients_match_oracle(native, count):
    p, x = _params(), _samples(count)
    grads = np.zeros(abi.MLP_PARAMS, np.float32)
    loss = C.c_double()
    native.check(native.lib.kgpu_mlp_gradients(
        native.handle, p.ctypes.data_as(C.POINTER(C.c_float)), x.ctypes.data_as(C.POINTER(C.c_float)),
        count, grads.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
    ref_loss, ref = loader.mlp_gradients(p, x, bf16_operands=True)
    assert abs(loss.value - ref_loss) <= 1e-5 * ref_loss
    for name, (lo, hi) in GROUPS.items():
        scale = np.max(np.abs(ref[lo:hi]))
        err = np.max(np.abs(grads[lo:hi] - ref[lo:hi]))
        assert err <= 1e-3 * scale + 1e-9, (name, err, scale)


def test_oracle_adam_first_step_and_descent():
    """The first Adam step moves every parameter with a nonzero gradient by the learning
    rate against the gradient's sign; a few hundred steps reduce the loss."""
    p, x = _params(), _samples(512)
    lr = 1e-3
    _, g = loader.mlp_gradients(p, x)
    one = loader.mlp_adam(p, x, 512, 1, lr)
    moved = np.abs(g) > 1e-4
    assert np.allclose((one - p)[moved], -lr * np.sign(g[moved]), rtol=1e-3, atol=1e-7)
    before, _ = loader.mlp_gradients(p, x)
    after, _ = loader.mlp_gradients(loader.mlp_adam(p, x, 128, 200, lr), x)
    assert after < 0.5 * before, (after, before)


@pytest.mark.gpu
@pytest.mark.parametrize("trainer", ["cluster", "grid"])
@pytest.mark.parametrize("count,batch,steps", [(1000, 1000, 1), (3000, 1024, 12), (20000, 8192, 6)])
def test_tensor_core_adam_matches_oracle(native, count, batch, steps, trainer):
    """kgpu_mlp_train (both tensor-core trainers: the clustered one, with its on-chip
    network and slice exchange, and the grid-barrier one) against the oracle's float32
    Adam on the oracle's gradients.  One
    step moves each parameter by the learning rate against the gradient's sign, so the
    parameters agree to rounding wherever the gradient is not negligible; over twelve
    steps the ratio m / sqrt(v) amplifies the 1e-3 relative gradient differences only for
    parameters whose gradient sits near zero, so 99% of the parameters agree to 2% of one
    step and all of them to one step per step."""
    lr = 1e-3
    p, x = _params(), _samples(count)
    got = p.copy()
    native.check(native.lib.kgpu_mlp_train(
        native.handle, got.ctypes.data_as(C.POINTER(C.c_float)), x.ctypes.data_as(C.POINTER(C.c_float)),
        count, batch, steps, lr, abi.TRAINER_CLUSTER if trainer == "cluster" else abi.TRAINER_GRID))
    ref = loader.mlp_adam(p, x, batch, steps, lr)
    diff = np.abs(got - ref)
    assert np.max(diff) <= lr * steps, np.max(diff)
    assert np.quantile(diff, 0.99) <= 0.02 * lr, np.quantile(diff, 0.99)
    ref_loss, _ = loader.mlp_gradients(ref, x)
    got_loss, _ = loader.mlp_gradients(got, x)
    assert abs(got_loss - ref_loss) <= 1e-3 * ref_loss, (got_loss, ref_loss)


def _heston():
    return PricingContext(HestonParameters(0.03, 0.0, 0.04, 2.0, 0.04, 0.5, -0.7), 100.0)


@pytest.mark.gpu
def test_mlp_lsmc_is_deterministic_and_near_the_adi_price(native, oracle):
    ctx = _heston()
    model = ctx.kgpu_model()
    adi = oracle.kor_heston_adi_american(C.byref(model), 100.0, -1.0, 1.0, 200, 50, 200, 1)
    s = lsmc_settings(1 << 15, 10, 42, abi.BASIS_MLP, precision="fp32", substeps=2)
    s.mlp_epochs, s.mlp_batch, s.mlp_learning_rate, s.mlp_seed = 3, 4096, 1e-3, 7
    a = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s, fresh_seed=43)
    b = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s, fresh_seed=43)
    assert a.price == b.price and a.out_of_sample == b.out_of_sample
    assert math.isfinite(a.price) and math.isfinite(a.out_of_sample)
    # In-sample LSMC is biased high, the out-of-sample policy low; both within a few
    # standard errors plus the 10-date discretisation of the exercise right.
    assert a.out_of_sample - 4 * a.out_of_sample_error < adi + 0.05
    assert abs(a.price - adi) < 0.25, (a.price, adi)


@pytest.mark.gpu
def test_network_improves_the_polynomial_exercise_policy(native):
    """The fitted network corrects the cubic polynomial's continuation value: on fresh
    paths (the same draws for both policies) its exercise policy is worth more, i.e. its
    out-of-sample lower bound is closer to the ADI price.  Training is deterministic, so
    this is a fixed comparison, not a statistical one."""
    ctx = _heston()
    poly = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0,
                    lsmc_settings(1 << 18, 10, 42, abi.BASIS_POLY3, precision="fp32", substeps=2),
                    fresh_seed=43)
    s = lsmc_settings(1 << 18, 10, 42, abi.BASIS_MLP, precision="fp32", substeps=2)
    s.mlp_epochs, s.mlp_batch, s.mlp_learning_rate, s.mlp_seed = 5, 8192, 1e-3, 7
    mlp = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s, fresh_seed=43)
    assert mlp.out_of_sample > poly.out_of_sample, (mlp.out_of_sample, poly.out_of_sample)


@pytest.mark.gpu
def test_standalone_network_prices_the_american_put(native, oracle):
    """The network alone (no polynomial, targets the discounted cash flows themselves) as
    the continuation estimate: deterministic, and its in-sample price and out-of-sample
    lower bound sit near the ADI price like the residual network's."""
    ctx = _heston()
    model = ctx.kgpu_model()
    adi = oracle.kor_heston_adi_american(C.byref(model), 100.0, -1.0, 1.0, 200, 50, 200, 1)
    s = lsmc_settings(1 << 16, 10, 42, abi.BASIS_MLP_STANDALONE, precision="fp32", substeps=2)
    s.mlp_epochs, s.mlp_batch, s.mlp_learning_rate, s.mlp_seed = 5, 4096, 1e-3, 7
    a = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s, fresh_seed=43)
    b = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s, fresh_seed=43)
    assert a.price == b.price and a.out_of_sample == b.out_of_sample
    assert a.out_of_sample - 4 * a.out_of_sample_error < adi + 0.05
    assert abs(a.price - adi) < 0.25, (a.price, adi)
    assert abs(a.out_of_sample - adi) < 0.25, (a.out_of_sample, adi)
