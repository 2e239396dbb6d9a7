"""The learned preconditioner on the GPU: the network's forward pass and
gradients from the hand-written kernels against the CPU oracle
(oracle/mlp_oracle.py), reproducibility, training, the chunk features of
bfgSystemLearnedPairs against the oracle's, and flexible GMRES with the
learned preconditioner against block-Jacobi alone."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import mlp_oracle as M

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import butterfly_gb300 as B  # noqa: E402
from butterfly_gb300 import learned as L  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return B.default_context(0)


def test_forward_and_gradients_match_oracle(ctx):
    shape = (96, 80, 40)        # not multiples of the 64-wide tiles
    net = L.Mlp(*shape, seed=3, context=ctx)
    rng = np.random.default_rng(1)
    X = rng.standard_normal((300, shape[0])).astype(np.float32)
    T = rng.standard_normal((300, shape[2])).astype(np.float32)
    p = net.get_params().astype(np.float64)
    Yo = M.forward(p, X.astype(np.float64), shape)[0]
    Y = net.forward(torch.from_numpy(X).cuda()).cpu().numpy()
    assert rel_err(Y, Yo) < 1e-5
    lo, go = M.loss_and_grad(p, X, T, shape)
    loss, g = net.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    assert abs(loss - lo) < 1e-5 * lo
    assert rel_err(g, go) < 1e-4
    # fixed-order reductions: the same batch, the same bits
    assert np.array_equal(g, net.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())[1])


def test_adam_step_matches_oracle_and_training_fits(ctx):
    shape = (16, 32, 8)
    net = L.Mlp(*shape, seed=4, context=ctx)
    rng = np.random.default_rng(2)
    X = torch.from_numpy(rng.standard_normal((512, 16)).astype(np.float32)).cuda()
    Wt = rng.standard_normal((16, 8)).astype(np.float32)
    T = X @ torch.from_numpy(Wt).cuda()                       # a linear map to learn
    p0 = net.get_params().astype(np.float64)
    _, g = M.loss_and_grad(p0, X.cpu().numpy(), T.cpu().numpy(), shape)
    net.train_step(X, T, 1e-3)
    p1o, _, _ = M.adam_step(p0, g, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
    assert rel_err(net.get_params(), p1o) < 1e-5
    losses = L.train(net, X, T, epochs=200, batch=128, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]


@pytest.fixture(scope="module")
def scattering(ctx):
    k = 40.0
    pts, nrm, w, off, _ = B.scattering_geometry(num=8, k=k, ppw=12, rmin=0.2, rmax=0.4,
                                                box=2.0, gap=0.1, seed=3)
    helm = B.Helm2(k, B.LayerPot.CombinedField, alpha=-1j * k, beta=1.0)
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm, leaf_size=32),
                                     B.Quadtree(pts, leaf_size=32), rank_eps=1e-10,
                                     pinv_tol=1e-10, context=ctx)
    system = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
    system.build_block_jacobi()
    return dict(pts=pts, off=off, system=system, k=k)


def test_learned_pairs_match_oracle(scattering):
    system, off = scattering["system"], scattering["off"]
    chunk = 16
    net = L.Mlp(4 * chunk, 64, 2 * chunk, seed=5)
    L.set_learned(system, net, chunk)
    n = len(scattering["pts"])
    rng = np.random.default_rng(3)
    r = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    e = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    F, T = L.learned_pairs(system, torch.from_numpy(r).cuda(), torch.from_numpy(e).cuda())
    zbj = system.apply_block_jacobi(torch.from_numpy(r).cuda()).cpu().numpy()
    Fo, To, _ = M.learned_pairs(r, zbj, e, off, chunk)
    # the solver's block-Jacobi runs from FP32 inverses, the public apply in FP64
    assert rel_err(F.cpu().numpy(), Fo) < 1e-5
    assert rel_err(T.cpu().numpy(), To) < 1e-5


def test_learned_fgmres_trained_on_own_solves(scattering):
    """Train on pairs from GMRES solves at 8 incident angles, solve at 2
    held-out angles with and without the network: both reach the tolerance
    with an FP64 true residual below it; the iteration counts are the
    network's measured gain (reported, not asserted: a per-chunk network
    sees only local residuals, while block-Jacobi already inverts each
    scatterer's self-interaction)."""
    system, pts, k = scattering["system"], scattering["pts"], scattering["k"]
    chunk = 16
    net = L.Mlp(4 * chunk, 256, 2 * chunk, seed=6)
    L.set_learned(system, net, chunk)
    Fs, Ts = [], []
    for i in range(8):
        th = 2 * np.pi * (i + 0.5) / 8
        b = torch.from_numpy(-np.exp(1j * k * (pts @ np.array([np.cos(th), np.sin(th)])))).cuda()
        F, T, _ = L.collect_pairs(system, b, iterates=(0, 5, 15))
        Fs.append(F)
        Ts.append(T)
    F, T = torch.cat(Fs), torch.cat(Ts)
    losses = L.train(net, F, T, epochs=60, batch=256, lr=1e-3)
    assert losses[-1] < losses[0]
    its = {}
    for th in (0.3, 2.2):
        b = torch.from_numpy(-np.exp(1j * k * (pts @ np.array([np.cos(th), np.sin(th)])))).cuda()
        for pc in ("block_jacobi", "learned"):
            x, info = B.solve_gmres(system, b, tol=1e-10, max_num_iter=400, precond=pc)
            assert info["converged"] == 1 and info["trueRelResidual"] < 1e-9
            its.setdefault(pc, []).append(info["iterations"])
    print("iterations block-Jacobi %s learned %s" % (its["block_jacobi"], its["learned"]))


def test_learned_rejects_a_network_of_the_wrong_shape(scattering):
    system = scattering["system"]
    net = L.Mlp(4 * 16, 32, 2 * 8, seed=1)         # output for 8 points, chunks of 16
    with pytest.raises(B.BfgError):
        L.set_learned(system, net, 16)
