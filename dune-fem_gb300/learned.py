"""Training and evaluation driver of the learned preconditioner.

Training pairs come from the solver itself, on seeded log-Gaussian kappa
fields (256 Fourier modes, std 1, correlation length 0.1):
  1. x* = the FP64-accurate solution of -div(kappa grad u) = 1 (SIPG, weak
     u = 0), from the mixed FP32/FP64 iterative refinement to 1e-10;
  2. iterates x_k of block-Jacobi PCG at k in `ks` (k = 0: x_0 = 0) give
     errors e_k = x* - x_k and residuals r_k = A e_k (FP64 apply);
  3. the network learns the part of e_k block Jacobi misses:
     target_k = e_k - BJ(r_k).
The network is then used as z = BJ(r) + NN(r) inside flexible CG, where the
FP64 residual decides convergence and block Jacobi is the fallback.
All compute runs in the library's CUDA kernels; this module only sequences
calls through the C-ABI.
"""
import time

import numpy as np

import gbfem


def sipg_problem(cells, order, seed, precision=gbfem.F64):
    """(op64, op32, kappa64, f): the variable-kappa SIPG problem of `seed`."""
    cl = (cells, cells, cells)
    modes = gbfem.fourier_modes(seed, 256, 0.1, 1.0)
    k64 = gbfem.project(cl, order, gbfem.FN_EXP_FOURIER, modes=modes)
    k32 = gbfem.convert(k64, gbfem.F32)
    op64 = gbfem.DGOperator(cl, order, kappa=k64)
    op32 = gbfem.DGOperator(cl, order, precision=gbfem.F32, kappa=k32)
    f = gbfem.project(cl, order, gbfem.FN_CONSTANT, params=(1.0,), scale_by_volume=True)
    return op64, op32, k64, k32, f


def _rms(x):
    return np.sqrt(max(gbfem.dot(x, x), 0.0) / x.n)


def make_pairs(cells, order, seed, ks=(0, 10, 40, 120, 400, 1000), inner_tol=1e-3, form="additive"):
    """Training pairs (r_k, target_k) in FP32 for one kappa seed, plus the kappa field.
    form "additive": target e_k - BJ(r_k); "twolevel": target e_k."""
    op64, op32, k64, k32, f = sipg_problem(cells, order, seed)
    bj32 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F32)   # blocks from the FP32 operator
    xs = gbfem.DeviceArray(op64.size)
    xs.clear()
    info = gbfem.solve_mixed(op64, op32, bj32, f, xs, tolerance=1e-10, inner_tolerance=inner_tol)
    if not info.converged:
        raise RuntimeError("make_pairs: reference solve did not converge (seed %d)" % seed)
    f32 = gbfem.convert(f, gbfem.F32)
    pairs = []
    for k in ks:
        inv = gbfem.KrylovInverseOperator("cg", tolerance=1e-12, max_iterations=k)
        inv.bind(op32, bj32)
        xk = gbfem.DeviceArray(op32.size, gbfem.F32)
        xk.clear()
        inv(f32, xk)
        e = gbfem.copy(xs)                      # e = x* - x_k (FP64)
        gbfem.axpy(-1.0, gbfem.convert(xk, gbfem.F64), e)
        r = gbfem.DeviceArray(op64.size)
        op64(e, r)                              # r = A e
        r32 = gbfem.convert(r, gbfem.F32)
        t = gbfem.convert(e, gbfem.F32)
        if form == "additive":                  # target = e - BJ(r)
            z = gbfem.DeviceArray(op32.size, gbfem.F32)
            bj32(r32, z)
            gbfem.axpy(-1.0, z, t)
        pairs.append((r32, t))
    return pairs, k32


def train(cnn, cells, order, seeds, ks=(0, 10, 40, 120, 400, 1000), steps_per_pair=4, lr=1e-3, log=None,
          form="additive"):
    """Online training over `seeds`; returns the per-step losses."""
    losses = []
    t0 = time.perf_counter()
    for i, seed in enumerate(seeds):
        pairs, k32 = make_pairs(cells, order, seed, ks, form=form)
        cnn.set_kappa(k32)
        if i == 0:
            r, t = pairs[-1]
            cnn.scale = _rms(t) / _rms(r)
        for _ in range(steps_per_pair):
            for r, t in pairs:
                losses.append(cnn.train_step(r, t, lr))
        if log:
            log("seed %d (%d/%d): loss %.4e  (%.1f s)" % (seed, i + 1, len(seeds), losses[-1],
                                                         time.perf_counter() - t0))
    return losses


def train_anorm(cnn, cells, order, seeds, ks=(0, 10, 40, 120, 400, 1000), steps_per_pair=4, lr=1e-3, log=None,
                form="additive"):
    """Online training with the energy-norm loss of the preconditioned step,
    L = (z - e)^T A (z - e) / e^T A e: the quantity that governs (flexible) CG
    convergence.  dL/dz = 2 A (z - e) / e^T A e costs one FP32 operator apply.
      additive:  z = BJ(r) + NN(r),             dL/dNN = dL/dz
      twolevel:  z = NN(r) + BJ(r - A NN(r)),   dL/dNN = (I - A BJ) dL/dz
    (BJ and A symmetric); in the two-level form the network runs in coarse
    mode (cell means in, cell means out): a learned coarse-grid correction."""
    losses = []
    t0 = time.perf_counter()
    for i, seed in enumerate(seeds):
        op64, op32, k64, k32, f = sipg_problem(cells, order, seed)
        del op64
        pairs, _ = make_pairs(cells, order, seed, ks, form="twolevel")   # (r, e) in FP32
        bj32 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F32)
        cnn.set_kappa(k32)
        if i == 0:
            r, e = pairs[0]
            cnn.scale = _rms(e) / _rms(r)
        twolevel = form == "twolevel"
        cnn.set_coarse(twolevel)
        pc = cnn.preconditioner(bj32, op32 if twolevel else None)
        n = op32.size
        z = gbfem.DeviceArray(n, gbfem.F32)
        ad = gbfem.DeviceArray(n, gbfem.F32)
        ae = gbfem.DeviceArray(n, gbfem.F32)
        t1 = gbfem.DeviceArray(n, gbfem.F32)
        t2 = gbfem.DeviceArray(n, gbfem.F32)
        for _ in range(steps_per_pair):
            for r, e in pairs:
                op32(e, ae)
                eae = gbfem.dot(e, ae)
                pc(r, z)                          # z = P(r)
                gbfem.axpy(-1.0, e, z)            # z <- z - e
                op32(z, ad)
                losses.append(gbfem.dot(z, ad) / eae)
                gbfem.check(gbfem.lib().gbfem_scal(gbfem.F32, n, 2.0 / eae, ad.ptr, None))   # g = dL/dz
                if twolevel:                      # dL/dNN = g - A BJ g
                    bj32(ad, t1)
                    op32(t1, t2)
                    gbfem.axpy(-1.0, t2, ad)
                cnn.train_step_grad(r, ad, lr)
        if log:
            log("seed %d (%d/%d): A-norm loss %.4e  (%.1f s)" % (seed, i + 1, len(seeds), losses[-1],
                                                                 time.perf_counter() - t0))
    return losses


def train_projected(cnn, cells, order, seeds, ks=(0, 10, 40, 120, 400, 1000), steps_per_pair=4, lr=1e-3, log=None):
    """Training for the two-level form with the Galerkin-scaled coarse
    correction (the network in coarse mode proposes the shape n of the
    error's cell means; the preconditioner uses alpha n, alpha = n.r / n.An):
    on the solver's own pairs (r_k, e_k), minimise
        L = 1 - (n.A e)^2 / ((n.A n)(e.A e)),
    the fraction of the A-norm error that the best multiple of n leaves.  L
    is invariant to the scale of n, so the network only has to learn where
    the smooth error is, not its size.  With a = n.r (= n.A e), b = n.A n:
        dL/dn = 2 a / (b E) (a / b A n - r),  E = e.A e.
    Returns the per-step losses."""
    losses = []
    t0 = time.perf_counter()
    cnn.set_coarse(True)
    for i, seed in enumerate(seeds):
        op64, op32, k64, k32, f = sipg_problem(cells, order, seed)
        del op64
        pairs, _ = make_pairs(cells, order, seed, ks, form="twolevel")   # (r, e) in FP32
        cnn.set_kappa(k32)
        n = op32.size
        z = gbfem.DeviceArray(n, gbfem.F32)
        az = gbfem.DeviceArray(n, gbfem.F32)
        ae = gbfem.DeviceArray(n, gbfem.F32)
        g = gbfem.DeviceArray(n, gbfem.F32)
        for _ in range(steps_per_pair):
            for r, e in pairs:
                op32(e, ae)
                E = gbfem.dot(e, ae)
                cnn.forward(r, z)                 # n = NN(r)
                op32(z, az)
                a, b = gbfem.dot(z, r), gbfem.dot(z, az)
                if not (b > 0.0 and E > 0.0):
                    continue
                losses.append(1.0 - a * a / (b * E))
                # g = 2 a / (b E) * (a / b * A n - r)
                g.clear()
                gbfem.axpy(a / b, az, g)
                gbfem.axpy(-1.0, r, g)
                gbfem.check(gbfem.lib().gbfem_scal(gbfem.F32, n, 2.0 * a / (b * E), g.ptr, None))
                cnn.train_step_grad(r, g, lr)
        if log:
            log("seed %d (%d/%d): projected loss %.4e  (%.1f s)" % (seed, i + 1, len(seeds), losses[-1] if losses
                                                                      else float("nan"), time.perf_counter() - t0))
    return losses


def evaluate(cnn, cells, order, seed, tol=1e-10, max_iterations=20000, plain=True, form="additive",
             plain_max_iterations=None, restart=20):
    """Iterations and times on one held-out seed: FP64 flexible CG with the
    learned preconditioner vs FP64 block-Jacobi PCG (and unpreconditioned CG),
    plus the mixed FP32/FP64 solve with the learned preconditioner inside.
    restart: directions the flexible CG keeps (the learned preconditioner is
    nonlinear, so a longer memory keeps more of CG's Krylov optimality)."""
    op64, op32, k64, k32, f = sipg_problem(cells, order, seed)
    out = {"seed": seed}
    bj64 = gbfem.Preconditioner.block_jacobi(op64)
    bj32 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F32)
    cnn.set_kappa(k64)
    cnn.set_coarse(form == "twolevel")
    learned64 = cnn.preconditioner(bj64, op64 if form == "twolevel" else None)
    u = gbfem.DeviceArray(op64.size)
    runs = [("bj_cg", "cg", bj64), ("learned_fcg", "fcg", learned64)]
    if plain:
        runs.insert(0, ("plain_cg", "cg", None))
    for name, method, pc in runs:
        cap = plain_max_iterations if (name == "plain_cg" and plain_max_iterations) else max_iterations
        inv = gbfem.KrylovInverseOperator(method, tolerance=tol, max_iterations=cap, restart=restart)
        inv.bind(op64, pc)
        u.clear()
        t0 = time.perf_counter()
        inv(f, u)
        i = inv.info()
        out[name] = {"iterations": i["iterations"], "time_s": time.perf_counter() - t0,
                     "converged": i["converged"], "fallbacks": i["fallbacks"]}
    # mixed precision + learned (FP32 inner flexible CG, FP64 refinement)
    learned32 = cnn.preconditioner(bj32, op32 if form == "twolevel" else None)
    for name, pc, method in (("mixed_bj", bj32, "cg"), ("mixed_learned", learned32, "fcg")):
        u.clear()
        t0 = time.perf_counter()
        info = gbfem.solve_mixed(op64, op32, pc, f, u, tolerance=tol, inner_method=method, inner_tolerance=1e-3,
                                 inner_restart=restart)
        out[name] = {"iterations": info.iterations, "time_s": time.perf_counter() - t0,
                     "converged": bool(info.converged), "rel_residual": info.residual}
    return out


def diagnose(cnn, cells, order, seed, ks=(0, 40, 400), form="additive"):
    """A-norm quality of the preconditioner on held-out solver pairs:
    ||e - z||_A / ||e||_A for z = BJ(r) and for the learned z."""
    op64, op32, k64, k32, f = sipg_problem(cells, order, seed)
    pairs, _ = make_pairs(cells, order, seed, ks, form="twolevel")   # targets = e
    bj32 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F32)
    cnn.set_kappa(k32)
    cnn.set_coarse(form == "twolevel")
    pc = cnn.preconditioner(bj32, op32 if form == "twolevel" else None)
    out = []
    for (r32, e), k in zip(pairs, ks):
        z = gbfem.DeviceArray(op32.size, gbfem.F32)
        bj32(r32, z)
        zn = gbfem.DeviceArray(op32.size, gbfem.F32)
        pc(r32, zn)
        res = {"k": k}
        for name, zz in (("bj", z), ("learned", zn)):
            d = gbfem.convert(e, gbfem.F64)
            gbfem.axpy(-1.0, gbfem.convert(zz, gbfem.F64), d)
            ad = gbfem.DeviceArray(op64.size)
            op64(d, ad)
            e64 = gbfem.convert(e, gbfem.F64)
            ae = gbfem.DeviceArray(op64.size)
            op64(e64, ae)
            res[name] = float(np.sqrt(gbfem.dot(d, ad) / gbfem.dot(e64, ae)))
        out.append(res)
    return out
