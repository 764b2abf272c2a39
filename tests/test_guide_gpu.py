"""GPU tests of the learned proposal's network (tcgen05 BF16 MLP, FP32
accumulation) against a plain PyTorch fp32 reference of the same network.

The kernels round the inputs, weights and every hidden activation to BF16
(the tensor-core operand type) and accumulate in FP32.  The reference does
the same roundings explicitly, so the remaining differences are summation
order and the rare activation that lands on the other side of a BF16
rounding boundary: lobe weights, log-concentrations and |m| |d mu| (the
direction error scaled by the length of the raw mean vector m, since m/|m|
is ill-conditioned for short m) agree to 2e-2 absolute, gradients to 3e-2
relative (norm of the difference over norm of the reference)."""
import math

import numpy as np
import pytest

from yar_gb300 import native

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

LOBE_ABS_TOL = 2e-2
GRAD_REL_TOL = 3e-2
LOSS_REL_TOL = 1e-2
BOX = (-1.0, 0.0, -1.5, 2.0, 2.5, 1.0)


def bf16(x):
    return x.to(torch.bfloat16).to(torch.float32)


def unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def random_rows(n, seed, train=False):
    rng = np.random.default_rng(seed)
    lo, hi = np.array(BOX[:3]), np.array(BOX[3:])
    rows = np.zeros((n, 16 if train else 12), np.float32)
    rows[:, 0:3] = lo + (hi - lo) * rng.random((n, 3))
    rows[:, 3:6] = unit(rng.normal(size=(n, 3)))
    rows[:, 6:9] = unit(rng.normal(size=(n, 3)))
    if train:
        rows[:, 9:12] = unit(rng.normal(size=(n, 3)))
        rows[:, 12] = rng.exponential(1.0, n)
    return rows


def random_params(seed, out_scale=0.5):
    rng = np.random.default_rng(seed)
    w1 = rng.uniform(-1, 1, (64, 128)) * math.sqrt(6 / 102)
    w2 = rng.uniform(-1, 1, (64, 64)) * math.sqrt(6 / 63)
    w3 = rng.uniform(-1, 1, (64, 64)) * math.sqrt(6 / 63)
    w4 = rng.uniform(-1, 1, (64, 64)) * math.sqrt(6 / 63) * out_scale
    w4[40:] = 0.0
    return np.concatenate([w.ravel() for w in (w1, w2, w3, w4)]).astype(np.float32)


def split(params):
    p = torch.as_tensor(params)
    return (p[0:8192].view(64, 128), p[8192:12288].view(64, 64), p[12288:16384].view(64, 64),
            p[16384:20480].view(64, 64))


def features(rows):
    r = torch.as_tensor(rows[:, 0:9], dtype=torch.float64)
    lo = torch.tensor(BOX[:3], dtype=torch.float64)
    hi = torch.tensor(BOX[3:], dtype=torch.float64)
    p = (r[:, 0:3] - lo) / (hi - lo)
    cols = []
    for k in range(16):  # f_k = (2^((k mod 3)/3) in float32) 2^(k div 3)
        s = float(np.float32(np.exp2(np.float64(k % 3) / 3.0))) * 2.0 ** (k // 3)
        for c in range(3):
            x = p[:, c].float().double() * s
            cols += [torch.sin(math.pi * x), torch.cos(math.pi * x)]
    x = torch.zeros(r.shape[0], 128, dtype=torch.float64)
    x[:, 0:96] = torch.stack(cols, 1)
    x[:, 96:102] = r[:, 3:9]
    x[:, 127] = 1.0
    return bf16(x.float())


def forward(params, rows, grad=False):
    w1, w2, w3, w4 = [bf16(w).clone().requires_grad_(grad) for w in split(params)]
    h = features(rows)

    def layer(h, w):
        a = h @ w.t()
        a = torch.cat([torch.relu(a[:, :63]), torch.ones_like(a[:, 63:])], 1)
        return a + (bf16(a) - a).detach()          # BF16 rounding with a straight-through gradient

    h1 = layer(h, w1)
    h2 = layer(h1, w2)
    h3 = layer(h2, w3)
    return h3 @ w4.t(), (w1, w2, w3, w4)


def mixture(o):
    m = o[:, 0:40].reshape(-1, 8, 5)
    mvec = m[:, :, 0:3]
    length = mvec.norm(dim=2, keepdim=True) + 1e-6
    mu = mvec / length
    kappa = torch.exp(torch.clamp(m[:, :, 3], -3.0, 8.0))
    logpi = torch.log_softmax(m[:, :, 4], 1)
    return mu, kappa, logpi


def log_q(o, d):
    mu, kappa, logpi = mixture(o)
    c = (mu * torch.as_tensor(d)[:, None, :]).sum(2)
    logc = torch.log(kappa) - math.log(2 * math.pi) - torch.log1p(-torch.exp(-2 * kappa))
    return torch.logsumexp(logpi + logc + kappa * (c - 1), 1)


def device(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def test_inference_matches_torch(gpu_ctx):
    params = random_params(3)
    gpu_ctx.guide_set_params(params)
    assert np.array_equal(gpu_ctx.guide_get_params(), params)
    for n in (1, 127, 128, 129, 5000):       # partial tiles, one tile, many tiles
        rows = random_rows(n, 10 + n)
        q = device(rows)
        lobes = torch.zeros((n, 40), dtype=torch.float32, device="cuda")
        gpu_ctx.guide_infer(q.data_ptr(), n, BOX, lobes.data_ptr())
        got = lobes.cpu().numpy().reshape(n, 8, 5)
        with torch.no_grad():
            o, _ = forward(params, rows)
            mu, kappa, logpi = mixture(o)
            mlen = o[:, 0:40].reshape(-1, 8, 5)[:, :, 0:3].norm(dim=2).numpy()
        want = torch.cat([mu, kappa[:, :, None], torch.exp(logpi)[:, :, None]], 2).numpy()
        # a lobe direction is m / |m|: its error is compared as |m| |d mu|, the
        # perpendicular change of the raw mean vector m
        err_mu = (np.abs(got[:, :, 0:3] - want[:, :, 0:3]).max(2) * mlen).max()
        err_k = np.abs(np.log(got[:, :, 3]) - np.log(want[:, :, 3])).max()
        err_pi = np.abs(got[:, :, 4] - want[:, :, 4]).max()
        assert err_mu < LOBE_ABS_TOL and err_k < LOBE_ABS_TOL and err_pi < LOBE_ABS_TOL, (n, err_mu, err_k, err_pi)
        assert np.allclose(got[:, :, 4].sum(1), 1.0, atol=1e-5)


def test_gradient_matches_torch(gpu_ctx):
    params = random_params(5)
    gpu_ctx.guide_set_params(params)
    n = 1000
    rows = random_rows(n, 21, train=True)
    scale = 0.7
    s = device(rows)
    grad = torch.zeros(native.GUIDE_PARAMS, dtype=torch.float32, device="cuda")
    loss = gpu_ctx.guide_gradient(s.data_ptr(), n, BOX, scale, grad.data_ptr())
    got = grad.cpu().numpy()
    o, ws = forward(params, rows, grad=True)
    w = torch.as_tensor(rows[:, 12]) * scale
    ref_loss = -(w * log_q(o, rows[:, 9:12])).sum()
    ref_loss.backward()
    ref = ref_loss.item()
    want = torch.cat([x.grad.ravel() for x in ws]).numpy()
    assert abs(loss - ref) <= LOSS_REL_TOL * abs(ref), (loss, ref)
    for name, sl in (("W1", slice(0, 8192)), ("W2", slice(8192, 12288)), ("W3", slice(12288, 16384)),
                     ("W4", slice(16384, 20480))):
        rel = np.linalg.norm(got[sl] - want[sl]) / np.linalg.norm(want[sl])
        assert rel < GRAD_REL_TOL, (name, rel)
    # unused parameters (bias-unit rows, outputs 40..63) receive no gradient
    assert np.all(got[16384 + 40 * 64: 20480] == 0.0)
    assert np.all(got[8192 + 63 * 64: 8192 + 64 * 64] == 0.0)


def test_training_concentrates_the_mixture(gpu_ctx):
    """Samples whose directions cluster around one axis: Adam steps on the
    tensor-core gradient must lower the loss and move the mixture's density
    there far above the uniform 1/(4 pi)."""
    gpu_ctx.guide_set_params(random_params(7, out_scale=0.1))
    n = 8192
    rows = random_rows(n, 31, train=True)
    rng = np.random.default_rng(32)
    target = np.array([0.3, 0.8, -0.52])
    target /= np.linalg.norm(target)
    rows[:, 9:12] = unit(target + 0.15 * rng.normal(size=(n, 3)))
    rows[:, 12] = 1.0
    s = device(rows)
    first = gpu_ctx.guide_train_step(s.data_ptr(), n, BOX, 1.0 / n, 5e-3)
    for _ in range(300):
        last = gpu_ctx.guide_train_step(s.data_ptr(), n, BOX, 1.0 / n, 5e-3)
    assert last < first - 2.0, (first, last)
    q = device(rows[:256, 0:12])
    lobes = torch.zeros((256, 40), dtype=torch.float32, device="cuda")
    gpu_ctx.guide_infer(q.data_ptr(), 256, BOX, lobes.data_ptr())
    lb = torch.as_tensor(lobes.cpu().numpy())
    mu, kappa, pi = lb.view(256, 8, 5)[:, :, 0:3], lb.view(256, 8, 5)[:, :, 3], lb.view(256, 8, 5)[:, :, 4]
    c = (mu * torch.as_tensor(target, dtype=torch.float32)).sum(2)
    dens = (pi * kappa / (2 * math.pi * (1 - torch.exp(-2 * kappa))) * torch.exp(kappa * (c - 1))).sum(1)
    assert float(dens.median()) > 10.0 / (4 * math.pi), float(dens.median())


def test_bounded_wait_gives_up_and_the_context_stays_usable(gpu_ctx):
    """The tensor-core kernels wait on mbarriers with an iteration limit.  A
    wait on a barrier that nothing arrives at (a 1000-poll test limit) must
    come back as YAR_ERR_TIMEOUT, and the next network call must work."""
    with pytest.raises(native.YarError) as e:
        gpu_ctx.wait_selftest(1000)
    assert e.value.code == native.YAR_ERR_TIMEOUT
    params = random_params(5)
    gpu_ctx.guide_set_params(params)
    n = 256
    q = device(random_rows(n, 77))
    lobes = torch.zeros((n, 40), dtype=torch.float32, device="cuda")
    gpu_ctx.guide_infer(q.data_ptr(), n, BOX, lobes.data_ptr())
    got = lobes.cpu().numpy().reshape(n, 8, 5)
    assert np.allclose(got[:, :, 4].sum(1), 1.0, atol=1e-5)
