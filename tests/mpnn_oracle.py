"""FP64 numpy restatement of the learned-guess network of
phase_gb300/csrc/mpnn.cu -- TEST INFRASTRUCTURE (gradient checks)."""
import numpy as np

H, F, L = 32, 4, 3


def layout():
    o = 0
    lay = {}
    def take(name, size):
        nonlocal o
        lay[name] = (o, size)
        o += size
    take("w0", F * H); take("b0", H)
    for l in range(L):
        take(f"P{l}", H * H); take(f"c{l}", H); take(f"U{l}", 2 * H * H); take(f"d{l}", H)
    take("wo", H); take("bo", 1)
    return lay, o


def round_bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even)."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def loss(params, rp, ci, a, b, xp, xs):
    lay, _ = layout()
    P = lambda k, shape: np.asarray(params[lay[k][0]:lay[k][0] + lay[k][1]],
                                    np.float64).reshape(shape)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    spmv = lambda x: np.bincount(rows, weights=a * x[ci], minlength=n)
    r = b - spmv(xp)
    diag = np.zeros(n)
    dmask = ci == rows
    diag[rows[dmask]] = a[dmask]
    e = np.where(dmask, 0.0, -a / diag[rows])
    sx = np.sqrt(np.mean(xp ** 2))
    sb = np.sqrt(np.mean(b ** 2))
    la = np.mean(np.log(np.abs(diag)))
    sd = np.sqrt(np.mean((r / diag) ** 2))
    f = np.stack([xp / sx, b / sb, r / sb, np.log(np.abs(diag)) - la], 1)
    relu = lambda z: np.maximum(z, 0.0)
    h = relu(f @ P("w0", (F, H)) + P("b0", (H,)))
    for l in range(L):
        q = h @ P(f"P{l}", (H, H)) + P(f"c{l}", (H,))
        m = np.zeros_like(h)
        np.add.at(m, rows, e[:, None] * relu(q[ci]))
        z = np.concatenate([h, m], 1) @ P(f"U{l}", (2 * H, H)) + P(f"d{l}", (H,))
        h = h + relu(z)
    out = h @ P("wo", (H,)) + P("bo", (1,))[0]
    g = xp + sd * out
    res = spmv(g) - b
    r0 = spmv(xp) - b
    return (res @ res) / (r0 @ r0) + ((g - xs) @ (g - xs)) / ((xp - xs) @ (xp - xs)), g
