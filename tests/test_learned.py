"""The learned preconditioner: GPU forward/backward kernels against the CPU
oracle (oracle/cnn_oracle.py), training, checkpoint/resume, and its use in
flexible CG with the block-Jacobi fallback."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("order,engine", [(1, "tensor"), (3, "tensor"), (3, "mma")])
def test_forward_and_gradients_match_cpu_oracle(gb, order, engine):
    import cnn_oracle as co
    N = 8
    nloc = (order + 1) ** 3
    net = gb.CNN(order, N, seed=3)
    net.set_conv_engine(engine)
    rng = np.random.default_rng(order)
    n = N ** 3 * nloc
    kappa = np.zeros(n)
    kappa[::nloc] = np.exp(rng.normal(0, 1, N ** 3))
    net.set_kappa(gb.DeviceArray.from_numpy(kappa))
    net.scale = 0.7
    r = rng.uniform(-1, 1, n)
    t = rng.uniform(-1, 1, n)
    dr, dt = gb.DeviceArray.from_numpy(r), gb.DeviceArray.from_numpy(t)
    z = gb.DeviceArray(n)
    net.forward(dr, z)
    Ws = co.unflatten(net.params(), nloc)
    logk = np.log(kappa[::nloc])
    loss_ref, g_ref, y = co.loss_grad(Ws, r, t, logk, N, nloc, 0.7)
    rms = np.sqrt(np.mean(r ** 2))
    z_ref = (0.7 * rms * y[:, :nloc]).ravel()
    # random weights: BF16 rounding of near-ties differs between the FP32
    # accumulation and the float64 oracle and propagates; measured worst over
    # orders 1-3 and two seeds: output 3e-3, loss 2e-6, 1 - cos 4e-4
    assert _rel(z.numpy(), z_ref) < 1e-2
    loss = net.loss_grad(dr, dt)
    assert abs(loss - loss_ref) < 1e-4 * loss_ref
    g = co.unflatten(net.grads(), nloc)
    for i, (a, b) in enumerate(zip(g, g_ref)):
        cos = np.sum(a * b) / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-300)
        assert cos > 0.998, (i, cos)
        assert _rel(a, b) < 0.1, (i, _rel(a, b))
    assert net.status() == 0


@pytest.mark.parametrize("order,engine,N", [(1, "tensor", 8), (3, "tensor", 8), (3, "mma", 8), (1, "tensor", 16)])
def test_exact_arithmetic_network_matches_oracle_bitwise(gb, order, engine, N):
    """With one tap per 3x3x3 layer and a scaled permutation as its channel
    matrix, weights in {1/2, 1, 2}, inputs +-1 (rms 1), kappa 1 and dyadic
    targets, every product and sum the kernels form is exact in FP32, so the
    GPU and the oracle round the same values to BF16: the output must agree
    bitwise and the weight gradients to FP32 accumulation order.  A wrong tap
    offset, flip or channel index anywhere in forward, backward-data or
    weight-gradient kernels shows as a mismatch."""
    import cnn_oracle as co
    nloc = (order + 1) ** 3
    net = gb.CNN(order, N, seed=1)
    net.set_conv_engine(engine)
    rng = np.random.default_rng(10 + order)
    shapes, cin0, cout0 = co.layer_shapes(nloc)
    Ws = []
    for li, (taps, cout, cin) in enumerate(shapes):
        W = np.zeros((taps, cout, cin))
        t = int(rng.integers(taps))
        src = rng.permutation(cin)[:cout] if cout <= cin else rng.integers(cin, size=cout)
        if li == 0:  # read the residual channels where there are enough of them
            src = rng.permutation(min(nloc, cin))[:cout] if nloc >= cout else src
        W[t, np.arange(cout), src] = rng.choice([0.5, 1.0, 2.0], size=cout)
        Ws.append(W)
    net.set_params(np.concatenate([W.ravel() for W in Ws]).astype(np.float32))
    n = N ** 3 * nloc
    kappa = np.zeros(n)
    kappa[::nloc] = 1.0
    net.set_kappa(gb.DeviceArray.from_numpy(kappa))
    net.scale = 1.0
    r = rng.choice([-1.0, 1.0], size=n)
    t = rng.integers(-8, 9, size=n) * 0.25
    dr, dt = gb.DeviceArray.from_numpy(r), gb.DeviceArray.from_numpy(t)
    z = gb.DeviceArray(n)
    net.forward(dr, z)
    loss_ref, g_ref, y = co.loss_grad(Ws, r, t, np.zeros(N ** 3), N, nloc, 1.0)
    z_ref = y[:, :nloc].ravel()
    assert np.max(np.abs(z_ref)) > 0
    assert np.array_equal(z.numpy(), z_ref)
    loss = net.loss_grad(dr, dt)
    assert abs(loss - loss_ref) <= 1e-6 * loss_ref
    g = co.unflatten(net.grads(), nloc)
    nonzero = 0
    for i, (a, b) in enumerate(zip(g, g_ref)):
        nonzero += int(np.count_nonzero(b))
        assert np.max(np.abs(a - b)) <= 1e-5 * max(np.max(np.abs(b)), 1e-30), (i, _rel(a, b))
    assert nonzero > 0
    assert net.status() == 0


def test_tensor_core_and_mma_convolutions_agree(gb):
    """Both engines on a 32^3 grid (256 tiles of 128 positions, two CTAs per
    SM): the outputs agree to the BF16 rounding of FP32 sums taken in a
    different order, and the training step's gradients likewise."""
    N, order = 32, 2
    nloc = 27
    n = N ** 3 * nloc
    rng = np.random.default_rng(5)
    kappa = np.zeros(n)
    kappa[::nloc] = np.exp(rng.normal(0, 1, N ** 3))
    r = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    t = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    outs, grads = [], []
    for engine in ("tensor", "mma"):
        net = gb.CNN(order, N, seed=7)
        net.set_conv_engine(engine)
        net.set_kappa(gb.DeviceArray.from_numpy(kappa))
        z = gb.DeviceArray(n)
        net.forward(r, z)
        net.loss_grad(r, t)
        outs.append(z.numpy())
        grads.append(net.grads())
        assert net.status() == 0
    assert _rel(outs[0], outs[1]) < 2e-2
    cos = np.dot(grads[0], grads[1]) / (np.linalg.norm(grads[0]) * np.linalg.norm(grads[1]))
    assert cos > 0.999


def test_training_reduces_the_loss_and_is_reproducible(gb):
    N, order = 8, 2
    n = N ** 3 * 27
    rng = np.random.default_rng(1)
    r = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, n).astype(np.float32))
    t = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, n).astype(np.float32))
    runs = []
    for _ in range(2):
        net = gb.CNN(order, N, seed=5)
        losses = [net.train_step(r, t, 3e-3) for _ in range(40)]
        runs.append((losses, net.params()))
    assert runs[0][0][-1] < 0.7 * runs[0][0][0]
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1])


def test_checkpoint_roundtrip_and_rejection(gb, tmp_path):
    net = gb.CNN(3, 8, seed=9)
    net.scale = 2.5
    path = str(tmp_path / "net.bin")
    net.save(path)
    other = gb.CNN(3, 8, seed=10)
    other.load(path)
    assert np.array_equal(other.params(), net.params()) and other.scale == 2.5
    data = bytearray(open(path, "rb").read())
    data[40:44] = np.array([np.nan], dtype=np.float32).tobytes()
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(bytes(data))
    with pytest.raises(gb.GbfemError):
        other.load(bad)
    with pytest.raises(gb.GbfemError):
        gb.CNN(2, 8).load(path)  # another space


def test_learned_fcg_certifies_and_falls_back_from_a_broken_network(gb):
    """A network with absurd weights must not spoil the solve: the FP64
    residual decides, flexible CG falls back to block Jacobi."""
    import learned
    cells, order = 16, 2
    op64, op32, k64, k32, f = learned.sipg_problem(cells, order, 123)
    bj = gb.Preconditioner.block_jacobi(op64)
    net = gb.CNN(order, cells, seed=1)
    net.set_kappa(k64)
    net.set_params(1e3 * np.random.default_rng(0).normal(size=net.num_params).astype(np.float32))
    net.scale = 1e6
    pc = net.preconditioner(bj)
    inv = gb.KrylovInverseOperator("fcg", tolerance=1e-10, max_iterations=5000, restart=4)
    inv.bind(op64, pc)
    u = gb.DeviceArray(op64.size)
    u.clear()
    inv(f, u)
    info = inv.info()
    assert info["converged"] and info["fallbacks"] >= 1
    r = gb.DeviceArray(op64.size)
    op64(u, r)
    x, ff = r.numpy(), f.numpy()
    assert np.linalg.norm(ff - x) <= 1.01e-10 * np.linalg.norm(ff)


def test_zero_network_reduces_both_forms_to_block_jacobi(gb):
    import learned
    cells, order = 8, 2
    op64, op32, k64, k32, f = learned.sipg_problem(cells, order, 5)
    bj = gb.Preconditioner.block_jacobi(op64)
    net = gb.CNN(order, cells, seed=2)
    net.set_kappa(k64)
    net.set_params(np.zeros(net.num_params, dtype=np.float32))
    r = gb.DeviceArray.from_numpy(np.random.default_rng(0).uniform(-1, 1, op64.size))
    zb, za, zt = (gb.DeviceArray(op64.size) for _ in range(3))
    bj(r, zb)
    net.preconditioner(bj)(r, za)
    net.preconditioner(bj, op64)(r, zt)
    assert np.array_equal(za.numpy(), zb.numpy())
    assert np.array_equal(zt.numpy(), zb.numpy())


def test_energy_norm_training_step_lowers_the_energy_loss(gb):
    """gbfem_cnn_train_step_grad with dL/dz = 2 A (z - e) / e^T A e."""
    import learned
    cells, order = 8, 2
    op64, op32, k64, k32, f = learned.sipg_problem(cells, order, 7)
    bj = gb.Preconditioner.block_jacobi(op32, gb.F32)
    n = op32.size
    rng = np.random.default_rng(1)
    e = gb.DeviceArray.from_numpy(rng.uniform(-1, 1, n).astype(np.float32))
    r = gb.DeviceArray(n, gb.F32)
    op32(e, r)
    net = gb.CNN(order, cells, seed=4)
    net.set_kappa(k32)
    pc = net.preconditioner(bj)
    z, ad, ae = (gb.DeviceArray(n, gb.F32) for _ in range(3))
    op32(e, ae)
    eae = gb.dot(e, ae)
    losses = []
    for _ in range(30):
        pc(r, z)
        gb.axpy(-1.0, e, z)
        op32(z, ad)
        losses.append(gb.dot(z, ad) / eae)
        gb.check(gb.lib().gbfem_scal(gb.F32, n, 2.0 / eae, ad.ptr, None))
        net.train_step_grad(r, ad, 1e-3)
    assert losses[-1] < 0.9 * losses[0]


def test_trained_network_gains_over_block_jacobi_on_held_out_kappa(gb):
    """What the trained network gains over the method without it.  16^3 DG
    Q2 SIPG, -div(kappa grad u) = 1 with log-Gaussian kappa: the network is
    trained on the GPU (train_projected: pairs (r_k, e_k) from the solver's
    own block-Jacobi CG iterates on 64 kappa seeds) and used as the
    Galerkin-scaled coarse correction z = alpha NN(r) + BJ(r - alpha A NN(r)).
    On a held-out seed, flexible CG(20) with it needs fewer iterations to 1e-10
    than block-Jacobi CG (measured 682 vs 858), and the mixed FP32-in-FP64
    solve with it fewer inner iterations than with block Jacobi (674 vs
    1417); every solution is certified by the FP64 residual.  Training is
    bitwise reproducible, so the counts are fixed for a given GPU."""
    import learned
    cells, order = 16, 2
    net = gb.CNN(order, cells, seed=2026)
    net.scale = 1.0
    losses = learned.train_projected(net, cells, order, list(range(64)), steps_per_pair=4, lr=1e-3)
    assert np.mean(losses[-24:]) < np.mean(losses[:24])
    ev = learned.evaluate(net, cells, order, 100000, plain=False, form="twolevel", restart=20)
    print("held-out iterations: BJ-CG %d, learned FCG(20) %d (fallbacks %d); mixed BJ %d, mixed learned %d" % (
        ev["bj_cg"]["iterations"], ev["learned_fcg"]["iterations"], ev["learned_fcg"]["fallbacks"],
        ev["mixed_bj"]["iterations"], ev["mixed_learned"]["iterations"]))
    for k in ("bj_cg", "learned_fcg", "mixed_bj", "mixed_learned"):
        assert ev[k]["converged"]
    assert ev["learned_fcg"]["iterations"] < 0.9 * ev["bj_cg"]["iterations"]
    assert ev["mixed_learned"]["iterations"] < 0.75 * ev["mixed_bj"]["iterations"]
    op64, op32, k64, k32, f = learned.sipg_problem(cells, order, 100000)
    bj = gb.Preconditioner.block_jacobi(op64)
    net.set_kappa(k64)
    inv = gb.KrylovInverseOperator("fcg", tolerance=1e-10, max_iterations=20000, restart=20)
    inv.bind(op64, net.preconditioner(bj, op64))
    u = gb.DeviceArray(op64.size)
    u.clear()
    inv(f, u)
    au = gb.DeviceArray(op64.size)
    op64(u, au)
    ff = f.numpy()
    assert np.linalg.norm(ff - au.numpy()) <= 1.01e-10 * np.linalg.norm(ff)


def test_integer_float_double_conversions_match_the_hardware(gb):
    """The elementwise kernels convert between binary32 and binary64 in
    integer arithmetic (csrc/convert.cuh); on 16M bit patterns, including
    values near the binary32 limits and rounding ties, the results equal the
    hardware's conversions bit for bit."""
    import ctypes as C
    bad = C.c_uint64(1)
    gb.check(gb.lib().gbfem_selftest_conversions(C.c_uint64(1 << 24), C.c_uint64(12345), C.byref(bad)))
    assert bad.value == 0
