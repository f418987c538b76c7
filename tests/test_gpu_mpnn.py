"""Learned preconditioner (dgc_mpnn_*, dgc_fpcg_solve): the CUDA forward pass,
loss and gradients agree with a float64 NumPy reference using the same BF16
weights; training lowers the loss; flexible PCG with the network reaches the
true FP64 residual and the same solution as block-Jacobi PCG."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

import mpnn_ref  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("act", ["relu", "linear"])
@pytest.mark.parametrize("kind", ["l2", "energy"])
def test_forward_loss_and_gradients_match_numpy(kind, act):
    m = meshes.jittered_square(4, 21)   # K = 32
    N, L, S = 2, 2, 2
    linear = act == "linear"
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    net = dg.MPNN(D, layers=L, seed=3)
    net.set_loss(dg.MPNN_LOSS_L2 if kind == "l2" else dg.MPNN_LOSS_ENERGY)
    K, Np, npi = D.K, D.Np, D.NpP
    nbr = dg.host_mesh(m, N)[1]
    rng = np.random.default_rng(5)
    x = rng.standard_normal((S * K, npi)).astype(np.float32)
    t = rng.standard_normal((S * K, npi)).astype(np.float32)
    x[:, Np:] = 0.0
    w = net.get_weights()
    assert w.size == net.num_params
    assert not np.any(w[-(npi * 64 + npi):])   # the output layer starts at zero
    w = (rng.standard_normal(w.size) * 0.2).astype(np.float32)   # every block then carries gradient
    net.set_weights(w)
    if linear:
        net.set_activation(dg.MPNN_ACT_LINEAR)   # zeroes the biases
        w = net.get_weights()
        assert not np.any(w[npi * 64:npi * 64 + 64])   # bin
    xd = torch.from_numpy(x).cuda().reshape(-1)
    td = torch.from_numpy(t).cuda().reshape(-1)
    loss, grad = net.train_step(xd, td, lr=0.0, want_grad=True)

    def spd(v):  # the FP64 SPD form on one native-layout field
        return D.spd(torch.from_numpy(np.ascontiguousarray(v).reshape(-1)).cuda()).cpu().numpy().reshape(K, npi)

    loss_ref, grad_ref = mpnn_ref.loss_and_grad(w, x.astype(np.float64), t.astype(np.float64), nbr, K, npi, Np, L,
                                                spd=spd if kind == "energy" else None, linear=linear)
    assert abs(loss - loss_ref) / loss_ref < 1e-5
    assert relerr(grad.cpu().numpy(), grad_ref) < 1e-4
    # per-parameter-block agreement (every block carries gradient)
    g = grad.cpu().numpy()
    o = 0
    for size in [64 * npi, 64] + [64 * 64, 64 * 64, 64] * L + [npi * 64, npi]:
        if linear and size in (64, npi) and not np.any(grad_ref[o:o + size]):
            assert not np.any(g[o:o + size]), o      # bias gradients held at zero
        else:
            assert relerr(g[o:o + size], grad_ref[o:o + size]) < 1e-3, o
        o += size
    y = net.forward(torch.from_numpy(x[:K]).cuda().reshape(-1)).cpu().numpy().reshape(K, npi)
    y_ref = mpnn_ref.forward(w, x[:K].astype(np.float64), nbr, K, npi, L, linear)[0]
    assert relerr(y, y_ref) < 1e-5
    if linear:  # a linear map: net(2x - x') = 2 net(x) - net(x')
        x2 = rng.standard_normal((K, npi)).astype(np.float32)
        x2[:, Np:] = 0.0
        f = lambda v: net.forward(torch.from_numpy(np.ascontiguousarray(v)).cuda().reshape(-1)).cpu().numpy()  # noqa
        lhs = f((2.0 * x[:K] - x2).astype(np.float32))
        assert relerr(lhs, 2.0 * f(x[:K]) - f(x2)) < 1e-5


def test_forward_many_tiles_matches_numpy():
    # K = 2048 nodes per sample, 3 samples: 48 tiles of the 128-node tensor-core
    # layer, a ragged last tile, 4 layers with random (non-zero) weights
    m = meshes.jittered_square(32, 23)
    N, L = 3, 4
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    net = dg.MPNN(D, layers=L, seed=4)
    K, Np, npi = D.K, D.Np, D.NpP
    nbr = dg.host_mesh(m, N)[1]
    rng = np.random.default_rng(6)
    w = (rng.standard_normal(net.num_params) * 0.15).astype(np.float32)
    net.set_weights(w)
    x = rng.standard_normal((K, npi)).astype(np.float32)
    x[:, Np:] = 0.0
    y = net.forward(torch.from_numpy(x).cuda().reshape(-1)).cpu().numpy().reshape(K, npi)
    y_ref = mpnn_ref.forward(w, x.astype(np.float64), nbr, K, npi, L)[0]
    assert relerr(y, y_ref) < 1e-5
    D.check()


def test_residual_correction_form_composes_as_documented():
    # M(r) = z0 + (|r'|/c) net(c r'/|r'|), r' = r - S z0, z0 = Binv r; the FP32 S
    # inside against the FP64 one here, hence the 1e-5 tolerance
    m = meshes.jittered_square(12, 31)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    net = dg.MPNN(D, layers=2, seed=8)
    base = dg.MPNN(D, layers=1, seed=0)          # zero output layer: M(r) = Binv r
    rng = np.random.default_rng(9)
    w = (rng.standard_normal(net.num_params) * 0.1).astype(np.float32)
    net.set_weights(w)
    net.set_correction(dg.MPNN_CORR_RESIDUAL)
    rv = np.zeros((D.K, D.NpP))
    rv[:, :D.Np] = rng.standard_normal((D.K, D.Np))
    r = torch.from_numpy(rv.reshape(-1)).cuda()
    z = net.precondition(r).cpu().numpy()
    z0 = base.precondition(r)
    rp = (r - D.spd(z0)).cpu().numpy()
    c = np.sqrt(D.K * D.Np)
    nr = np.linalg.norm(rp)
    y = net.forward(torch.from_numpy((rp * c / nr).astype(np.float32)).cuda()).double().cpu().numpy()
    ref = z0.cpu().numpy() + y * nr / c
    ref.reshape(D.K, D.NpP)[:, D.Np:] = 0.0
    assert relerr(z, ref) < 1e-5
    assert relerr(z, z0.cpu().numpy()) > 1e-3      # the network term is present
    D.check()


def test_weights_round_trip_and_adam_step_moves_weights():
    m = meshes.jittered_square(3, 2)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    net = dg.MPNN(D, layers=1, seed=7)
    w = net.get_weights()
    net.set_weights(w * 0.5)
    assert np.array_equal(net.get_weights(), w * 0.5)
    x = torch.randn(D.K * D.NpP, device="cuda")
    t = torch.randn(D.K * D.NpP, device="cuda")
    net.train_step(x, t, lr=1e-3)
    assert not np.array_equal(net.get_weights(), w * 0.5)


def smooth_fields(x, y, count, rng, modes=6):
    out = []
    for _ in range(count):
        f = np.zeros_like(x)
        for _ in range(modes):
            kx, ky = rng.integers(1, 5, size=2)
            f += rng.normal() / (kx * kx + ky * ky) * np.sin(kx * np.pi * (x + 1) / 2) * np.sin(ky * np.pi * (y + 1) / 2)
        out.append(f.reshape(-1))
    return out


def test_training_lowers_loss_on_residual_error_pairs():
    m = meshes.jittered_square(8, 4)   # K = 128
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    net = dg.MPNN(D, layers=2, seed=1)
    net.set_loss(dg.MPNN_LOSS_L2)
    x, y = D.node_xy()
    rng = np.random.default_rng(0)
    xs, ts = [], []
    zero = dg.MPNN(D, layers=1, seed=0)
    zero.set_weights(np.zeros(zero.num_params, np.float32))   # M(r) = Binv r
    for e in smooth_fields(x, y, 8, rng):
        E = D.upload(e)
        r = D.spd(E)
        nr = float(torch.linalg.norm(r))
        bj = zero.precondition(r)
        xs.append((r / nr).float())
        ts.append(((E - bj) / nr).float())
    X, T = torch.cat(xs), torch.cat(ts)
    first, _ = net.train_step(X, T, lr=0.0)
    for _ in range(150):
        last, _ = net.train_step(X, T, lr=2e-3)
    assert last < 0.7 * first


def poisson_rhs(D):
    x, y = D.node_xy()
    f = 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)
    return D.mass(D.upload(f.reshape(-1)))


@pytest.mark.parametrize("window", [1, 4])
def test_fcg_with_zero_network_is_block_jacobi_pcg(window):
    m = meshes.jittered_square(8, 9)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, mode=dg.SOLVE_FP64_PCG, rtol=1e-10, graph=False)
    net = dg.MPNN(D, layers=1, seed=0)   # zero output layer: M = Binv
    xf, stf = net.fpcg(b, rtol=1e-10, window=window)
    assert stf["converged"] and stf["final_relres"] <= 1e-10
    # the same Krylov method in exact arithmetic; rounding moves the count a little
    assert abs(stf["iterations"] - stp["iterations"]) <= max(2, 0.05 * stp["iterations"])
    assert relerr(D.download(xf), D.download(xp)) < 1e-8


def test_fcg_with_random_network_reaches_true_residual():
    m = meshes.jittered_square(8, 9)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, mode=dg.SOLVE_FP64_PCG, rtol=1e-10)
    net = dg.MPNN(D, layers=4, seed=11)
    rng = np.random.default_rng(2)
    net.set_weights((rng.standard_normal(net.num_params) * 0.1).astype(np.float32))
    xf, stf = net.fpcg(b, rtol=1e-10, maxit=20 * stp["iterations"])
    assert stf["converged"] and stf["final_relres"] <= 1e-10
    assert relerr(D.download(xf), D.download(xp)) < 1e-8
    D.check()


def test_mpnn_needs_dirichlet_laplace():
    m = meshes.jittered_square(3, 3)
    with pytest.raises(dg.DgcError):
        dg.MPNN(dg.Discretization(m, "maxwell_te", 3, dg.F32))
    with pytest.raises(dg.DgcError):
        dg.MPNN(dg.Discretization(m, "laplace", 3, dg.F64, dirichlet=False))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_learned_solve_falls_back_to_block_jacobi_pcg(mode):
    m = meshes.jittered_square(8, 9)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, rtol=1e-10)
    net = dg.MPNN(D, layers=2, seed=4)
    rng = np.random.default_rng(8)
    net.set_weights((rng.standard_normal(net.num_params) * 0.1).astype(np.float32))
    md = dg.SOLVE_FP64_PCG if mode == "fp64" else dg.SOLVE_MIXED_IR
    x, st = net.solve(b, rtol=1e-10, fcg_maxit=5, mode=md)   # budget far too small: falls back
    assert st["fell_back"] and st["converged"] and st["final_relres"] <= 1e-10
    assert st["inner_iterations"] == 5 and st["iterations"] > 5
    assert relerr(D.download(x), D.download(xp)) < 1e-8


def test_learned_solve_without_fallback_when_budget_suffices():
    m = meshes.jittered_square(8, 9)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    _, stp = D.pcg(b, rtol=1e-10)
    net = dg.MPNN(D, layers=2, seed=4)   # zero output layer: flexible CG = block-Jacobi PCG
    x, st = net.solve(b, rtol=1e-10, fcg_maxit=2 * stp["iterations"])
    assert not st["fell_back"] and st["converged"] and st["final_relres"] <= 1e-10
    assert st["iterations"] == st["inner_iterations"]


def test_fcg_independent_of_stale_device_memory():
    """Work vectors start at zero and S u writes its padding: a flexible CG run
    after NaN-filled memory went back to the driver behaves as in a fresh process."""
    junk = torch.full((256 << 20,), float("nan"), dtype=torch.float32, device="cuda")
    del junk
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    m = meshes.jittered_square(8, 9)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, mode=dg.SOLVE_FP64_PCG, rtol=1e-10, graph=False)
    net = dg.MPNN(D, layers=1, seed=0)
    xf, stf = net.fpcg(b, rtol=1e-10, window=4)
    assert stf["converged"] and abs(stf["iterations"] - stp["iterations"]) <= max(2, 0.05 * stp["iterations"])
    assert relerr(D.download(xf), D.download(xp)) < 1e-8
