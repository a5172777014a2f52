"""CPU (numpy, float64) restatement of the learned preconditioner's network,
forward and backward, for checking the GPU kernels' outputs and gradients.

TEST INFRASTRUCTURE ONLY.  Forward and backward round every stored
activation and activation gradient to BF16 at the points where the GPU
stores BF16 (csrc/cnn.cu cnn_forward/cnn_backward); sums and products are
float64 in between, where the GPU accumulates in FP32.

Layer order and weight layout ([taps][cout][cin], tap t = (dz+1)*9 +
(dy+1)*3 + (dx+1)) follow the GPU network: in-proj 1x1 + relu, then
3x3x3 convs on levels N, N/2, N/4, N/8 with 2x2x2 average pooling, nearest
upsampling with skip addition, and a 1x1 out-proj.
"""
import numpy as np

C = 32


def bf16(a):
    """Round float32 values to BF16 (nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layer_shapes(nloc):
    cin0 = 32 if nloc + 1 <= 32 else (80 if nloc + 1 <= 80 else 128)
    cout0 = 32 if nloc <= 32 else (64 if nloc <= 64 else 128)
    shapes = [(1, C, cin0)] + [(27, C, C)] * 7 + [(1, cout0, C)]
    return shapes, cin0, cout0


def unflatten(flat, nloc):
    shapes, _, _ = layer_shapes(nloc)
    out, off = [], 0
    for s in shapes:
        n = s[0] * s[1] * s[2]
        out.append(np.asarray(flat[off:off + n], dtype=np.float64).reshape(s))
        off += n
    return out


def _grid(x, N):
    return x.reshape(N, N, N, -1)  # [z][y][x][c]


def conv(x, W, N):
    """out[p][co] = sum_{t,ci} W[t][co][ci] x[nbr(p,t)][ci], zero padding."""
    T = W.shape[0]
    g = _grid(x, N)
    if T == 1:
        return x @ W[0].T
    pad = np.zeros((N + 2, N + 2, N + 2, g.shape[3]))
    pad[1:-1, 1:-1, 1:-1] = g
    out = np.zeros((N, N, N, W.shape[1]))
    for t in range(27):
        dx, dy, dz = t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1
        sl = pad[1 + dz:1 + dz + N, 1 + dy:1 + dy + N, 1 + dx:1 + dx + N]
        out += sl @ W[t].T
    return out.reshape(N ** 3, -1)


def conv_bwd(x, W, dout, N):
    """(dx, dW) of out = conv(x, W)."""
    T = W.shape[0]
    if T == 1:
        return dout @ W[0], (dout.T @ x)[None]
    g = _grid(x, N)
    pad = np.zeros((N + 2, N + 2, N + 2, g.shape[3]))
    pad[1:-1, 1:-1, 1:-1] = g
    dpad = np.zeros_like(pad)
    do = _grid(dout, N)
    dW = np.zeros_like(W)
    for t in range(27):
        dx, dy, dz = t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1
        sl = (slice(1 + dz, 1 + dz + N), slice(1 + dy, 1 + dy + N), slice(1 + dx, 1 + dx + N))
        dW[t] = do.reshape(-1, W.shape[1]).T @ pad[sl].reshape(-1, W.shape[2])
        dpad[sl] += do @ W[t]
    return dpad[1:-1, 1:-1, 1:-1].reshape(N ** 3, -1), dW


def pool(x, N):
    g = _grid(x, N)
    M = N // 2
    return g.reshape(M, 2, M, 2, M, 2, -1).mean(axis=(1, 3, 5)).reshape(M ** 3, -1)


def pool_bwd(d, N):
    M = N // 2
    g = d.reshape(M, 1, M, 1, M, 1, -1) / 8.0
    return np.broadcast_to(g, (M, 2, M, 2, M, 2, g.shape[-1])).reshape(N ** 3, -1)


def up(x, N):
    """nearest upsampling from N/2 to N"""
    M = N // 2
    g = x.reshape(M, 1, M, 1, M, 1, -1)
    return np.broadcast_to(g, (M, 2, M, 2, M, 2, g.shape[-1])).reshape(N ** 3, -1)


def up_bwd(d, N):
    M = N // 2
    return d.reshape(M, 2, M, 2, M, 2, -1).sum(axis=(1, 3, 5)).reshape(M ** 3, -1)


relu = lambda a: np.maximum(a, 0.0)


def forward(Ws, r, logk, N, nloc):
    """Returns (y [P][cout0], cache); r is the dof vector, logk per cell."""
    Wb = [bf16(W) for W in Ws]
    _, cin0, cout0 = layer_shapes(nloc)
    P = N ** 3
    rms = np.sqrt(np.mean(np.asarray(r, np.float64) ** 2))
    x0 = np.zeros((P, cin0))
    x0[:, :nloc] = np.asarray(r, np.float64).reshape(P, nloc) / rms
    x0[:, nloc] = logk
    x0 = bf16(x0)
    L = [N, N // 2, N // 4, N // 8]
    c = {"x0": x0}
    c["a0"] = bf16(relu(conv(x0, Wb[0], L[0])))
    c["s1"] = bf16(relu(conv(c["a0"], Wb[1], L[0])))
    c["p1"] = bf16(pool(c["s1"], L[0]))
    c["s2"] = bf16(relu(conv(c["p1"], Wb[2], L[1])))
    c["p2"] = bf16(pool(c["s2"], L[1]))
    c["s3"] = bf16(relu(conv(c["p2"], Wb[3], L[2])))
    c["p3"] = bf16(pool(c["s3"], L[2]))
    c["b4"] = bf16(relu(conv(c["p3"], Wb[4], L[3])))
    c["u3"] = bf16(up(c["b4"], L[2]) + c["s3"])
    c["d3"] = bf16(relu(conv(c["u3"], Wb[5], L[2])))
    c["u2"] = bf16(up(c["d3"], L[1]) + c["s2"])
    c["d2"] = bf16(relu(conv(c["u2"], Wb[6], L[1])))
    c["u1"] = bf16(up(c["d2"], L[0]) + c["s1"])
    c["d1"] = bf16(relu(conv(c["u1"], Wb[7], L[0])))
    y = conv(c["d1"], Wb[8], L[0])
    c["Wb"], c["rms"], c["L"] = Wb, rms, L
    return y, c


def loss_grad(Ws, r, target, logk, N, nloc, S):
    """MSE loss of the GPU definition and the weight gradients (list, layer order)."""
    y, c = forward(Ws, r, logk, N, nloc)
    P = N ** 3
    t = np.zeros_like(y)
    t[:, :nloc] = np.asarray(target, np.float64).reshape(P, nloc) / (S * c["rms"])
    diff = y - t
    diff[:, nloc:] = 0.0
    loss = np.sum(diff ** 2) / (P * nloc)
    dy = bf16(2.0 * diff / (P * nloc))
    Wb, L = c["Wb"], c["L"]
    g = [None] * 9
    dd1, g[8] = conv_bwd(c["d1"], Wb[8], dy, L[0])
    dd1 = bf16(dd1) * (c["d1"] > 0)
    du1, g[7] = conv_bwd(c["u1"], Wb[7], dd1, L[0])
    du1 = bf16(du1)
    dd2 = bf16(up_bwd(du1, L[0]) * (c["d2"] > 0))
    du2, g[6] = conv_bwd(c["u2"], Wb[6], dd2, L[1])
    du2 = bf16(du2)
    dd3 = bf16(up_bwd(du2, L[1]) * (c["d3"] > 0))
    du3, g[5] = conv_bwd(c["u3"], Wb[5], dd3, L[2])
    du3 = bf16(du3)
    db4 = bf16(up_bwd(du3, L[2]) * (c["b4"] > 0))
    dp3, g[4] = conv_bwd(c["p3"], Wb[4], db4, L[3])
    ds3 = bf16((du3 + pool_bwd(bf16(dp3), L[2])) * (c["s3"] > 0))
    dp2, g[3] = conv_bwd(c["p2"], Wb[3], ds3, L[2])
    ds2 = bf16((du2 + pool_bwd(bf16(dp2), L[1])) * (c["s2"] > 0))
    dp1, g[2] = conv_bwd(c["p1"], Wb[2], ds2, L[1])
    ds1 = bf16((du1 + pool_bwd(bf16(dp1), L[0])) * (c["s1"] > 0))
    da0, g[1] = conv_bwd(c["a0"], Wb[1], ds1, L[0])
    da0 = bf16(da0) * (c["a0"] > 0)
    _, g[0] = conv_bwd(c["x0"], Wb[0], da0, L[0])
    return loss, g, y
