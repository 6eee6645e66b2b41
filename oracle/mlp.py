"""CPU restatement of the pair-energy surrogate (test infrastructure only).

Used by the tests to check the GPU surrogate: pose features (frames, minimum-image
centre vector, relative quaternion) and the MLP's forward pass, loss and gradients,
in float64.  With ``bf16=True`` the restatement rounds to bfloat16 where the GPU path
stores bfloat16 (weights of layers 2-4, hidden activations, activation gradients), so
that GPU results can be compared at a tolerance set by float32 accumulation rather than
by bfloat16 storage; with ``bf16=False`` it is the exact float64 network.

The surrogate has no counterpart in the reference; the pair energy it learns is the
reference's inter-molecule energy (src/Replica.cpp:502-528 E(a,b), src/Potential.cpp).
"""
import numpy as np

N_IN = 8
H = 256
POS_SCALE = 1.0 / 20.0
INV_SCALE = 10.0

_LAYOUT = (("W1", H * N_IN), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H), ("W4", H * H),
           ("b4", H), ("w5", H), ("b5", 1))
OFF = {}
_o = 0
for _k, _n in _LAYOUT:
    OFF[_k] = (_o, _n)
    _o += _n
N_PARAMS = _o


def bf16(x):
    """Round float values to bfloat16 (nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    rnd = ((bits >> 16) & 1) + 0x7FFF
    out = ((bits + rnd) & 0xFFFF0000).astype(np.uint32).view(np.float32)
    return out.astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(flat):
    p = {}
    for k, (o, n) in OFF.items():
        v = np.asarray(flat[o:o + n], np.float64)
        if k == "W1":
            v = v.reshape(H, N_IN)
        elif k in ("W2", "W3", "W4"):
            v = v.reshape(H, H)
        p[k] = v
    return p


def forward(flat, X, bf16_path=False):
    """Network output for rows X[n][8] and the cache the backward pass needs."""
    p = unpack(flat)
    r = bf16 if bf16_path else (lambda v: np.asarray(v, np.float64))
    X = np.asarray(X, np.float64)
    Z = [X @ p["W1"].T + p["b1"]]
    Hs = [r(silu(Z[0]))]
    for l in (2, 3, 4):
        W = r(p["W%d" % l])
        Z.append(Hs[-1] @ W.T + p["b%d" % l])
        Hs.append(r(silu(Z[-1])))
    o = Hs[-1] @ p["w5"] + p["b5"][0]
    return o, (p, X, Z, Hs)


def loss_grad(flat, X, y, bf16_path=False):
    """Mean squared error and its gradient (flat, in the parameter layout)."""
    o, (p, X, Z, Hs) = forward(flat, X, bf16_path)
    r = bf16 if bf16_path else (lambda v: np.asarray(v, np.float64))
    n = len(o)
    res = o - np.asarray(y, np.float64)
    loss = float(np.mean(res * res))
    dO = 2.0 * res / n
    g = {"w5": Hs[3].T @ dO, "b5": np.array([dO.sum()])}
    dZ = r(np.outer(dO, p["w5"]) * silu_grad(Z[3]))
    for l in (4, 3, 2):
        g["W%d" % l] = dZ.T @ Hs[l - 2]
        g["b%d" % l] = dZ.sum(0)
        W = r(p["W%d" % l])
        dZ = r((dZ @ W) * silu_grad(Z[l - 2]))
    g["W1"] = dZ.T @ X
    g["b1"] = dZ.sum(0)
    flat_g = np.zeros(N_PARAMS)
    for k, (o_, n_) in OFF.items():
        flat_g[o_:o_ + n_] = np.asarray(g[k]).reshape(-1)
    return loss, flat_g


# ------------------------------------------------------------------ pose features

def frame(q0, q1, q2):
    """Rows e1, e2, e3 of the Gram-Schmidt frame of three points."""
    a = np.asarray(q1, np.float64) - q0
    a = a / np.linalg.norm(a)
    b = np.asarray(q2, np.float64) - q0
    b = b - np.dot(a, b) * a
    b = b / np.linalg.norm(b)
    return np.array([a, b, np.cross(a, b)])


def quaternion(R):
    """Unit quaternion (w, x, y, z), w >= 0, of a rotation matrix (largest-component branch)."""
    t = np.trace(R)
    if t > 0:
        s = np.sqrt(t + 1.0) * 2
        q = [0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s]
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = np.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        q = [(R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s]
    elif R[1, 1] > R[2, 2]:
        s = np.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        q = [(R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s]
    else:
        s = np.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        q = [(R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s]
    q = np.array(q)
    return -q if q[0] < 0 else q


def features(Fa, ca, Fb, cb, box):
    d = np.asarray(cb, np.float64) - np.asarray(ca, np.float64)
    if box > 0:
        d = d - box * np.round(d / box)
    r = np.linalg.norm(d)
    x = np.zeros(N_IN)
    x[:3] = (Fa @ d) * POS_SCALE
    x[3] = INV_SCALE / max(r, 1.0)
    x[4:] = quaternion(Fa @ Fb.T)
    return x


def frame_residues(rel):
    """The three residues spanning a molecule's body frame (engine's choice)."""
    q = np.asarray(rel, np.float64)
    f0 = int(np.argmax((q * q).sum(1)))
    f1 = int(np.argmax(((q - q[f0]) ** 2).sum(1)))
    u = q[f1] - q[f0]
    u = u / np.linalg.norm(u)
    v = q - q[f0]
    perp = v - np.outer(v @ u, u)
    f2 = int(np.argmax((perp * perp).sum(1)))
    return f0, f1, f2
