"""Skin-scheduler network: the hand-written CUDA forward / backward / Adam kernels against a
float64 numpy restatement of the same 12 -> 64 -> 64 -> 2 SiLU network, and the restatement's
analytic gradient against central finite differences (CPU)."""
import numpy as np
import pytest

N_IN, N_H, N_OUT = 12, 64, 2
SIZES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("W3", (N_OUT, N_H)),
         ("b3", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(w):
    out, k = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = w[k:k + n].reshape(shp)
        k += n
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, X):
    p = unpack(w)
    z1 = X @ p["W1"].T + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = silu(z2)
    return h2 @ p["W3"].T + p["b3"], (z1, h1, z2, h2)


def loss_grad(w, X, T, ow):
    """Loss = mean over samples and outputs of ow[o] * (y - T)^2, and its gradient."""
    n = X.shape[0]
    p = unpack(w)
    y, (z1, h1, z2, h2) = forward(w, X)
    diff = y - T
    loss = float(np.sum(ow * diff * diff) / (n * N_OUT))
    dy = 2.0 * ow * diff / (n * N_OUT)
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dz2 = (dy @ p["W3"]) * silu_grad(z2)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"]) * silu_grad(z1)
    g["W1"] = dz1.T @ X
    g["b1"] = dz1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SIZES])


def init(rng):
    parts = []
    for name, shp in SIZES:
        if name.startswith("W"):
            parts.append(rng.normal(0, 1.0 / np.sqrt(shp[1]), size=shp).ravel())
        else:
            parts.append(rng.normal(0, 0.1, size=shp))
    return np.concatenate(parts)


def sample(rng, n):
    X = rng.normal(0, 1, size=(n, N_IN))
    T = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1], np.cos(X[:, 2]) * X[:, 3]], axis=1)
    return X, T


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = init(rng)
    X, T = sample(rng, 7)
    ow = np.array([1.0, 0.5])
    _, g = loss_grad(w, X, T, ow)
    idx = rng.choice(N_PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (loss_grad(wp, X, T, ow)[0] - loss_grad(wm, X, T, ow)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_parameter_count(gpu_lib):
    assert gpu_lib.mlp_num_params() == N_PARAMS  # no device call


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.gpu
def test_forward_and_gradient_match_reference(gpu_lib, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(1)
    w = init(rng)
    n = 1000  # several blocks of 32 samples, the last one ragged
    X, T = sample(rng, n)
    ow = np.array([1.0, 0.25])
    dev = torch.device("cuda:0")
    f32 = lambda a: torch.tensor(np.asarray(a, dtype=np.float32), device=dev)
    wt, Xt, Tt, owt = f32(w), f32(X), f32(T), f32(ow)
    Y = torch.zeros(n, N_OUT, device=dev)
    gpu_lib.mlp_forward(wt, Xt, Y)
    torch.cuda.synchronize()
    y_ref, _ = forward(w.astype(np.float32).astype(np.float64), X.astype(np.float32).astype(np.float64))
    np.testing.assert_allclose(Y.cpu().numpy(), y_ref, rtol=1e-4, atol=1e-5)

    ws = torch.zeros(gpu_lib.mlp_workspace_floats(n), device=dev)
    grad = torch.zeros(N_PARAMS, device=dev)
    loss = torch.zeros(1, device=dev)
    gpu_lib.mlp_grad(wt, Xt, Tt, owt, ws, grad, loss)
    torch.cuda.synchronize()
    l_ref, g_ref = loss_grad(w.astype(np.float32).astype(np.float64), X.astype(np.float32).astype(np.float64),
                             T.astype(np.float32).astype(np.float64), ow)
    g = grad.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - l_ref) <= 1e-5 * abs(l_ref)
    # norm-wise relative error of the whole gradient, and per block of parameters
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)
    k = 0
    for name, shp in SIZES:
        m = int(np.prod(shp))
        blk, ref = g[k:k + m], g_ref[k:k + m]
        assert np.linalg.norm(blk - ref) <= 1e-4 * np.linalg.norm(ref) + 1e-9, name
        k += m
    # deterministic: the block partials are summed in a fixed order
    grad2 = torch.zeros_like(grad)
    gpu_lib.mlp_grad(wt, Xt, Tt, owt, ws, grad2, loss)
    torch.cuda.synchronize()
    assert torch.equal(grad, grad2)


@pytest.mark.gpu
def test_adam_step_matches_reference(gpu_lib, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(2)
    dev = torch.device("cuda:0")
    w = rng.normal(size=N_PARAMS).astype(np.float32)
    g = rng.normal(size=N_PARAMS).astype(np.float32)
    m = rng.normal(size=N_PARAMS).astype(np.float32) * 0.1
    v = np.abs(rng.normal(size=N_PARAMS)).astype(np.float32) * 0.01
    t, lr = 3, 1e-3
    wt, gt, mt, vt = (torch.tensor(a, device=dev) for a in (w, g, m, v))
    gpu_lib.mlp_adam(wt, gt, mt, vt, t, lr)
    torch.cuda.synchronize()
    # the kernel's constants are FP32: 0.999f and 1 - 0.999f differ from 0.999 by ~1e-8
    f32 = np.float32
    b1, b2, eps = float(f32(0.9)), float(f32(0.999)), 1e-8
    c1, c2 = float(f32(1) - f32(0.9)), float(f32(1) - f32(0.999))
    m1 = b1 * m.astype(np.float64) + c1 * g
    v1 = b2 * v.astype(np.float64) + c2 * g.astype(np.float64) ** 2
    w1 = w - lr * (m1 / (1 - b1**t)) / (np.sqrt(v1 / (1 - b2**t)) + eps)
    np.testing.assert_allclose(mt.cpu().numpy(), m1, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(vt.cpu().numpy(), v1, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(wt.cpu().numpy(), w1, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_training_reduces_loss(gpu_lib, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(3)
    dev = torch.device("cuda:0")
    X, T = sample(rng, 512)
    Xt = torch.tensor(X.astype(np.float32), device=dev)
    Tt = torch.tensor(T.astype(np.float32), device=dev)
    ow = torch.ones(N_OUT, device=dev)
    w = torch.tensor(init(rng).astype(np.float32), device=dev)
    m, v = torch.zeros_like(w), torch.zeros_like(w)
    ws = torch.zeros(gpu_lib.mlp_workspace_floats(512), device=dev)
    grad, loss = torch.zeros_like(w), torch.zeros(1, device=dev)
    losses = []
    for t in range(1, 301):
        gpu_lib.mlp_grad(w, Xt, Tt, ow, ws, grad, loss)
        gpu_lib.mlp_adam(w, grad, m, v, t, 3e-3)
        if t in (1, 300):
            losses.append(float(loss.item()))
    assert losses[1] < 0.2 * losses[0], losses
