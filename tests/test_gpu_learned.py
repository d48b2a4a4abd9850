"""The learned part: the GPU MLP kernels against the float64 NumPy oracle
(forward, loss and gradients), training, and parareal with the identity and
with the learned coarse propagator, measured against the serial FP64 DG."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import mlp_oracle as M

pytestmark = pytest.mark.gpu

C0, RHO0 = 340.0, 1.225


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("nin,width,nout,hidden,rows", [(40, 64, 12, 3, 300), (37, 70, 13, 2, 301),
                                                         (261, 256, 80, 3, 517)])
def test_mlp_forward_loss_and_gradients_match_oracle(nin, width, nout, hidden, rows):
    rng = np.random.default_rng(nin)
    net = D.MLP(nin, width, nout, hidden, seed=3)
    net.set_gemm("simt")
    p = net.params()
    assert p.size == sum(o * i + o for (o, i) in M.shapes(nin, width, nout, hidden))
    p = (rng.standard_normal(p.size) * 0.2).astype(np.float32)
    net.set_params(p)
    X = rng.standard_normal((rows, nin)).astype(np.float32)
    T = rng.standard_normal((rows, nout)).astype(np.float32)
    Y = net.forward(X)
    Yo, _, _ = M.forward(p, X, nin, width, nout, hidden)
    assert rel(Y, Yo) <= 1e-5
    loss, g = net.loss_grad(X, T)
    lo, go = M.loss_grad(p, X, T, nin, width, nout, hidden)
    assert abs(loss - lo) <= 1e-5 * lo
    assert rel(g, go) <= 1e-4
    net.close()


@pytest.mark.parametrize("nin,width,nout,hidden,rows", [(40, 64, 12, 3, 300), (37, 70, 13, 2, 1000),
                                                         (261, 256, 80, 3, 517), (8, 16, 3, 1, 128)])
def test_mlp_bf16_tensor_core_inference(nin, width, nout, hidden, rows):
    """tcgen05 BF16 inference against its NumPy emulation (BF16 inputs,
    weights and hidden activations; a hidden value rounding the other way at
    a BF16 tie bound is the only difference) and against FP32 inference."""
    rng = np.random.default_rng(nin + rows)
    net = D.MLP(nin, width, nout, hidden, seed=5)
    p = (rng.standard_normal(net.params().size) * 0.2).astype(np.float32)
    net.set_params(p)
    X = rng.standard_normal((rows, nin)).astype(np.float32)
    Y = net.forward(X, bf16=True)
    Ye = M.forward_bf16(p, X, nin, width, nout, hidden)
    Yf = net.forward(X)
    assert rel(Y, Ye) <= 2e-3, rel(Y, Ye)
    assert rel(Y, Yf) <= 3e-2, rel(Y, Yf)
    # new weights reach the BF16 copy
    net.set_params(p * 0.5)
    Y2 = net.forward(X, bf16=True)
    assert rel(Y2, M.forward_bf16(p * 0.5, X, nin, width, nout, hidden)) <= 2e-3
    # deterministic
    assert np.array_equal(net.forward(X, bf16=True), Y2)
    net.close()


def test_mlp_training_reduces_the_loss():
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (2048, 6)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], X[:, 2] ** 2 - X[:, 3] * X[:, 4]], axis=1).astype(np.float32)
    net = D.MLP(6, 64, 2, 3, seed=1)
    first = net.loss_grad(X, T)[0]
    for _ in range(300):
        net.train_step(X, T, 3e-3)
    assert net.loss_grad(X, T)[0] < 0.05 * first


def room(nx=6, ny=5, nz=4, order=3):
    mesh = D.Mesh.box_tet(nx, ny, nz, (0.0, 0.0, 0.0), (1.2, 1.0, 0.8), order=order,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Reflecting", "Absorbing",
                                      "Reflecting"))
    return mesh, D.Precomp(mesh)


def test_identity_parareal_reaches_the_serial_dg_in_n_iterations():
    mesh, pre = room(4, 3, 3, order=2)
    dt = D.cfl_dt(pre, C0)
    u0 = pre.initial_state([(0, 0.5, 0.4, 0.4, 0.01, 1.0)])
    nslices, steps = 4, 5
    s = D.Solver(pre, C0, RHO0, flux="upwind")
    s.set_state(u0)
    s.rk4_steps(0.0, dt, nslices * steps)
    ref = s.get_state()
    out, iters, hist = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=0.0, max_iter=nslices)
    assert iters == nslices and len(hist) == nslices
    for q in range(4):
        assert rel(out[q], ref[q]) <= 1e-12
    # fewer iterations than slices leave the last slice inexact
    out2, _, _ = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=0.0, max_iter=2)
    assert rel(out2[0], ref[0]) > 1e-3


def test_learned_coarse_propagator_beats_the_identity():
    """Trained on FP64 DG trajectories of four pulse positions, the network
    (3 hidden GELU layers of 128, one fine step per application, energy
    clipped) propagates a pulse at a fifth position; parareal with it is
    closer to the serial DG after two iterations than parareal without it
    (identity coarse propagator), and converged parareal is the DG answer."""
    mesh, pre = room()
    dt = D.cfl_dt(pre, C0)
    L = D.Learned(pre, C0, RHO0, width=128, hidden_layers=3, coarse_steps=1, dt=dt, seed=7)
    for pos in [(0.3, 0.3, 0.3), (0.9, 0.7, 0.5), (0.5, 0.2, 0.6), (0.8, 0.5, 0.2)]:
        L.collect(pre.initial_state([(0, *pos, 0.02, 1.0)]), nsnap=60)
    assert L.num_samples() > 1000
    loss = L.train(epochs=40, batch=1024, lr=1e-3)
    assert np.isfinite(loss)
    u0 = pre.initial_state([(0, 0.6, 0.45, 0.4, 0.02, 1.0)])
    nslices, steps = 8, 16
    s = D.Solver(pre, C0, RHO0, flux="upwind")
    s.set_state(u0)
    s.rk4_steps(0.0, dt, nslices * steps)
    ref = s.get_state()
    err = {}
    for name, lrn in (("learned", L), ("identity", None)):
        out, it, _ = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=0.0, max_iter=2, learned=lrn)
        err[name] = rel(out[0], ref[0])
    assert err["learned"] < 0.5 * err["identity"], err
    st = L.step_stats()
    assert st["applications"] > 0 and 0.0 < st["alpha_mean"] <= 1.0
    # converged parareal with the network is the DG answer
    out, it, hist = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=1e-5, max_iter=nslices, learned=L)
    assert rel(out[0], ref[0]) <= 1e-4
    assert it <= nslices
    # and after as many iterations as slices it is the serial DG to rounding
    # (needs a bit-reproducible coarse step: G(U) - G(U) cancels exactly)
    out, it, _ = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=0.0, max_iter=nslices, learned=L)
    assert it == nslices
    for q in range(4):
        assert rel(out[q], ref[q]) <= 1e-11


def test_bf16_inference_in_the_coarse_propagator():
    """The coarse propagator with tensor-core BF16 inference: close to its
    FP32 inference, bit-reproducible, and parareal with it still reaches the
    serial DG after N iterations."""
    mesh, pre = room(4, 3, 3)
    dt = D.cfl_dt(pre, C0)
    L = D.Learned(pre, C0, RHO0, width=128, hidden_layers=3, coarse_steps=1, dt=dt, seed=2)
    u0 = pre.initial_state([(0, 0.5, 0.5, 0.4, 0.02, 1.0)])
    L.collect(u0, nsnap=20)
    L.train(epochs=5, batch=512)
    a32 = L.apply(u0, 4)
    L.set_inference("bf16")
    a16 = L.apply(u0, 4)
    assert np.array_equal(a16, L.apply(u0, 4))
    assert rel(a16[0], a32[0]) <= 2e-2
    nslices, steps = 4, 5
    s = D.Solver(pre, C0, RHO0, flux="upwind")
    s.set_state(u0)
    s.rk4_steps(0.0, dt, nslices * steps)
    ref = s.get_state()
    out, it, _ = D.parareal(pre, C0, RHO0, u0, nslices, steps, dt, tol=0.0, max_iter=nslices, learned=L)
    assert it == nslices
    for q in range(4):
        assert rel(out[q], ref[q]) <= 1e-11


def test_learned_coarse_step_is_bit_reproducible():
    mesh, pre = room(4, 3, 3)
    dt = D.cfl_dt(pre, C0)
    L = D.Learned(pre, C0, RHO0, width=64, hidden_layers=2, coarse_steps=1, dt=dt, seed=1)
    u0 = pre.initial_state([(0, 0.5, 0.5, 0.4, 0.02, 1.0)])
    L.collect(u0, nsnap=10)
    L.train(epochs=2, batch=512)
    a = L.apply(u0, 5)
    b = L.apply(u0, 5)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("nin,width,nout,hidden,rows", [(40, 64, 12, 3, 300), (37, 70, 13, 2, 301),
                                                         (261, 256, 80, 3, 517), (261, 256, 80, 3, 4096)])
@pytest.mark.parametrize("mode", ["tc", "simt"])
def test_training_gemms_on_both_paths_match_oracle(nin, width, nout, hidden, rows, mode):
    """The training GEMMs (forward, activation gradient, weight gradient over
    the rows, split over CTAs when the rows are many) on the tensor cores
    (3xTF32 split products, FP32 accumulation: the default) and on the CUDA
    cores: inference and gradients against the float64 oracle at the same
    bars (1e-5, 1e-4).  The loss is held to 1e-5 on
    the CUDA cores and 5e-5 on the tensor cores: their FP32 accumulation
    across the K-steps of an output (rounded per MMA) measured 1.3e-5 on the
    width-256 network with outputs of magnitude ~40.  A few Adam steps on
    either path stay within 1e-4 of the other."""
    rng = np.random.default_rng(nin + rows)
    net = D.MLP(nin, width, nout, hidden, seed=7)
    net.set_gemm(mode)
    p = (rng.standard_normal(net.params().size) * 0.2).astype(np.float32)
    net.set_params(p)
    X = rng.standard_normal((rows, nin)).astype(np.float32)
    T = rng.standard_normal((rows, nout)).astype(np.float32)
    Y = net.forward(X)
    Yo, _, _ = M.forward(p, X, nin, width, nout, hidden)
    assert rel(Y, Yo) <= 1e-5, rel(Y, Yo)
    loss, g = net.loss_grad(X, T)
    lo, go = M.loss_grad(p, X, T, nin, width, nout, hidden)
    assert abs(loss - lo) <= (5e-5 if mode == "tc" else 1e-5) * lo, (loss, lo)
    assert rel(g, go) <= 1e-4, rel(g, go)
    # a few Adam steps move both paths the same way
    other = D.MLP(nin, width, nout, hidden, seed=7)
    other.set_gemm("simt" if mode == "tc" else "tc")
    other.set_params(p)
    for _ in range(3):
        net.train_step(X, T, 1e-3)
        other.train_step(X, T, 1e-3)
    assert rel(net.params(), other.params().astype(np.float64)) <= 1e-4
    net.close()
    other.close()
