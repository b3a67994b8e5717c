"""FP64 numpy reference of the learned preconditioner's MLP (the checker for
the GPU training and inference kernels).

Parameters (15361 floats): W1[64][108], b1[64], W2[64][64], b2[64],
W3[64][64], b3[64], w4[64], b4.  Features per node: residual / patch RMS
[0,27), a_ij/a_ii [27,54), mask [54,81), a_jj/a_ii [81,108); the static part
is features 27..107.  GELU in its tanh form.  The stencil of a node is the
MLP on the 27 unit-impulse residuals (rms 1/sqrt 27, so the residual feature
is sqrt 27 at slot s), divided by sqrt 27 and masked; the training prediction
is rf_13 + sum_s c_s rf_s.
"""
import numpy as np

SQ27 = np.sqrt(27.0)
NP = 15361
SL = {"W1": (0, (64, 108)), "b1": (6912, (64,)), "W2": (6976, (64, 64)), "b2": (11072, (64,)),
      "W3": (11136, (64, 64)), "b3": (15232, (64,)), "w4": (15296, (64,)), "b4": (15360, (1,))}
K0 = np.sqrt(2.0 / np.pi)


def unpack(P):
    P = np.asarray(P, np.float64)
    return {k: P[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in SL.items()}


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K0 * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    th = np.tanh(K0 * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * K0 * (1.0 + 3 * 0.044715 * x * x)


def forward(P, st):
    """Activations of the impulse evaluation for static features st [n,81]."""
    w = unpack(P)
    st = np.asarray(st, np.float64)
    hs = st @ w["W1"][:, 27:].T + w["b1"]
    z1 = hs[:, None, :] + SQ27 * w["W1"][:, :27].T[None, :, :]
    h1 = gelu(z1)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = gelu(z2)
    z3 = h2 @ w["W3"].T + w["b3"]
    h3 = gelu(z3)
    o = h3 @ w["w4"] + w["b4"][0]
    return dict(w=w, st=st, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, o=o)


def stencil(P, st):
    f = forward(P, st)
    return f["st"][:, 27:54] * f["o"] / SQ27


def loss_and_grad(P, st, rf, tg):
    f = forward(P, st)
    w = f["w"]
    rf = np.asarray(rf, np.float64)
    tg = np.asarray(tg, np.float64)
    n = tg.size
    mask = f["st"][:, 27:54]
    c = mask * f["o"] / SQ27
    pred = rf[:, 13] + (c * rf).sum(1)
    diff = pred - tg
    loss = (diff ** 2).mean()
    dO = (2.0 * diff / n)[:, None] * rf * mask / SQ27
    g = {}
    g["w4"] = np.einsum("bs,bsk->k", dO, f["h3"])
    g["b4"] = np.array([dO.sum()])
    d3 = dO[:, :, None] * w["w4"][None, None, :] * gelu_grad(f["z3"])
    g["W3"] = np.einsum("bso,bsk->ok", d3, f["h2"])
    g["b3"] = d3.sum((0, 1))
    d2 = (d3 @ w["W3"]) * gelu_grad(f["z2"])
    g["W2"] = np.einsum("bso,bsk->ok", d2, f["h1"])
    g["b2"] = d2.sum((0, 1))
    d1 = (d2 @ w["W2"]) * gelu_grad(f["z1"])
    gW1 = np.zeros((64, 108))
    gW1[:, :27] = SQ27 * d1.sum(0).T
    dhs = d1.sum(1)
    gW1[:, 27:] = dhs.T @ f["st"]
    g["W1"] = gW1
    g["b1"] = dhs.sum(0)
    out = np.zeros(NP)
    for k, (o, s) in SL.items():
        out[o:o + int(np.prod(s))] = np.asarray(g[k]).ravel()
    return loss, out


def random_params(seed, out_scale=0.3):
    rng = np.random.default_rng(seed)
    P = np.zeros(NP)
    for k, (o, s) in SL.items():
        fan = s[1] if len(s) == 2 else (108 if k == "b1" else 64)
        P[o:o + int(np.prod(s))] = rng.uniform(-1, 1, int(np.prod(s))) / np.sqrt(fan)
    o, _ = SL["w4"]
    P[o:o + 65] *= out_scale * np.sqrt(64)
    return P


def random_samples(n, seed):
    """Feature rows with the ranges a continuity stencil produces."""
    rng = np.random.default_rng(seed)
    mask = (rng.uniform(size=(n, 27)) > 0.15).astype(np.float64)
    mask[:, 13] = 1.0
    st = np.concatenate([rng.uniform(-0.4, 0.05, (n, 27)) * mask, mask, rng.uniform(0.6, 1.6, (n, 27)) * mask], 1)
    st[:, 13] = 1.0
    st[:, 54 + 13] = 1.0
    rf = rng.normal(size=(n, 27)) * mask
    rf /= np.sqrt((rf ** 2).sum(1, keepdims=True) / 27)
    tg = rf[:, 13] + rng.normal(scale=0.3, size=n)
    return st, rf, tg


def slot_map(conn, n):
    """nbr[i][s]: neighbour of node i at element-local offset slot s (min index), -1 if none."""
    cs = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    nbr = np.full((n, 27), np.iinfo(np.int64).max, np.int64)
    for a in range(8):
        for b in range(8):
            d = cs[b] - cs[a] + 1
            code = 9 * d[2] + 3 * d[1] + d[0]
            np.minimum.at(nbr[:, code], conn[:, a], conn[:, b].astype(np.int64))
    nbr[nbr == np.iinfo(np.int64).max] = -1
    return nbr


def static_features(rp, ci, v, nbr):
    """[n,81] float32 static features from a CRS matrix (FP64 ratios rounded once)."""
    n = rp.size - 1
    diag = np.zeros(n)
    rows = np.repeat(np.arange(n), np.diff(rp))
    dmask = ci == rows
    diag[rows[dmask]] = v[dmask]
    dinv = np.where(diag != 0, 1.0 / np.where(diag != 0, diag, 1.0), 1.0)
    st = np.zeros((n, 81))
    for i in range(n):
        cols = ci[rp[i]:rp[i + 1]]
        vals = v[rp[i]:rp[i + 1]]
        for s in range(27):
            j = nbr[i, s]
            if j < 0:
                continue
            k = np.nonzero(cols == j)[0]
            aij = vals[k[0]] if k.size else 0.0
            st[i, s] = aij * dinv[i]
            st[i, 27 + s] = 1.0
            st[i, 54 + s] = dinv[i] / dinv[j]
    return st.astype(np.float32), dinv
