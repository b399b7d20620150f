"""CPU oracle of the coupling-layer normalizing flow (test infrastructure only).

Restates, in float64 numpy, the flow the engine trains and samples on the GPU
(graniitti_gb300/csrc/grn_flow.cu), so that the GPU forward pass, log-density,
inverse and parameter gradients can be checked. The method is the
rational-quadratic neural spline flow of Durkan, Bekasov, Murray, Papamakarios
(NeurIPS 2019) on the unit hypercube with affine-free coupling layers
(Dinh et al. 2017):

  density direction x -> z, layer l: z_A = x_A, z_B = RQS(x_B; theta_l(x_A)),
  log q(x) = sum_l sum_{j in B_l} log dRQS/dx  (z uniform on [0,1]^D),
  theta_l = MLP(x_A): D/2 -> H -> relu -> H -> relu -> (D/2)(3K+1).

Parameter layout per layer (row-major, weights stored [in][out]):
  W1 [D/2][H], b1 [H], W2 [H][H], b2 [H], W3 [H][(D/2)(3K+1)], b3 [(D/2)(3K+1)]
and per transformed dimension j the 3K+1 outputs are (K widths, K heights, K+1
derivatives). The GPU computes the matrix products from BF16-rounded weights and
activations with FP32 accumulation; `bf16=True` reproduces that rounding here.
"""
import numpy as np

MIN_W = 1e-3
MIN_H = 1e-3
MIN_D = 1e-3


def masks(dim):
    """Conditioning (A) and transformed (B) index sets of the six masks; layer l uses
    mask l % 6 (D = 8, 12 or 14): halves, even / odd, neighbour pairs, each then swapped."""
    if dim == 8:
        A = [[0, 1, 2, 3], [4, 5, 6, 7], [0, 2, 4, 6], [1, 3, 5, 7], [0, 1, 4, 5], [2, 3, 6, 7]]
    elif dim == 12:
        A = [list(range(6)), list(range(6, 12)), list(range(0, 12, 2)), list(range(1, 12, 2)),
             [0, 1, 4, 5, 8, 9], [2, 3, 6, 7, 10, 11]]
    elif dim == 14:
        A = [list(range(7)), list(range(7, 14)), list(range(0, 14, 2)), list(range(1, 14, 2)),
             [0, 1, 4, 5, 8, 9, 12], [2, 3, 6, 7, 10, 11, 13]]
    else:
        raise ValueError("flow masks exist for D = 8, 12 and 14")
    return [(a, [j for j in range(dim) if j not in a]) for a in A]


def n_out(dim, bins):
    return (dim // 2) * (3 * bins + 1)


def layer_sizes(dim, hidden, bins):
    a = dim // 2
    o = n_out(dim, bins)
    return [("W1", (a, hidden)), ("b1", (hidden,)), ("W2", (hidden, hidden)), ("b2", (hidden,)),
            ("W3", (hidden, o)), ("b3", (o,))]


def n_params(dim, layers, hidden, bins):
    return layers * sum(int(np.prod(s)) for _, s in layer_sizes(dim, hidden, bins))


def unpack(theta, dim, layers, hidden, bins):
    """Flat parameter vector -> list of per-layer dicts (views)."""
    out, k = [], 0
    for _ in range(layers):
        d = {}
        for name, shape in layer_sizes(dim, hidden, bins):
            n = int(np.prod(shape))
            d[name] = theta[k:k + n].reshape(shape)
            k += n
        out.append(d)
    return out


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def softplus(x):
    return np.logaddexp(0.0, x)


def spline_params(raw, bins):
    """raw (n, 3K+1) -> knots X, Y (n, K+1), derivatives d (n, K+1)."""
    K = bins
    wr, hr, dr = raw[:, :K], raw[:, K:2 * K], raw[:, 2 * K:]
    w = np.exp(wr - wr.max(1, keepdims=True))
    w = MIN_W + (1 - K * MIN_W) * w / w.sum(1, keepdims=True)
    h = np.exp(hr - hr.max(1, keepdims=True))
    h = MIN_H + (1 - K * MIN_H) * h / h.sum(1, keepdims=True)
    d = MIN_D + softplus(dr)
    X = np.concatenate([np.zeros((len(raw), 1)), np.cumsum(w, 1)], 1)
    Y = np.concatenate([np.zeros((len(raw), 1)), np.cumsum(h, 1)], 1)
    X[:, -1] = 1.0
    Y[:, -1] = 1.0
    return X, Y, d


def rqs_forward(x, raw, bins):
    """y = RQS(x) and log dy/dx, x (n,) in [0,1]."""
    X, Y, d = spline_params(raw, bins)
    n = len(x)
    k = np.clip(np.sum(X[:, 1:-1] <= x[:, None], 1), 0, bins - 1)
    r = np.arange(n)
    xk, wk = X[r, k], X[r, k + 1] - X[r, k]
    yk, hk = Y[r, k], Y[r, k + 1] - Y[r, k]
    dk, dk1 = d[r, k], d[r, k + 1]
    s = hk / wk
    xi = (x - xk) / wk
    om = xi * (1 - xi)
    den = s + (dk1 + dk - 2 * s) * om
    y = yk + hk * (s * xi * xi + dk * om) / den
    dydx = s * s * (dk1 * xi * xi + 2 * s * om + dk * (1 - xi) ** 2) / (den * den)
    return y, np.log(dydx)


def rqs_inverse(y, raw, bins):
    """x = RQS^{-1}(y) (Durkan et al. eq. 6-8)."""
    X, Y, d = spline_params(raw, bins)
    n = len(y)
    k = np.clip(np.sum(Y[:, 1:-1] <= y[:, None], 1), 0, bins - 1)
    r = np.arange(n)
    xk, wk = X[r, k], X[r, k + 1] - X[r, k]
    yk, hk = Y[r, k], Y[r, k + 1] - Y[r, k]
    dk, dk1 = d[r, k], d[r, k + 1]
    s = hk / wk
    dy = y - yk
    a = hk * (s - dk) + dy * (dk1 + dk - 2 * s)
    b = hk * dk - dy * (dk1 + dk - 2 * s)
    c = -s * dy
    xi = 2 * c / (-b - np.sqrt(b * b - 4 * a * c))
    return xk + xi * wk


def conditioner(xa, p, bf=True):
    q = bf16 if bf else (lambda v: v)
    h1 = np.maximum(q(xa) @ q(p["W1"]) + p["b1"], 0.0)
    h2 = np.maximum(q(h1) @ q(p["W2"]) + p["b2"], 0.0)
    return q(h2) @ q(p["W3"]) + p["b3"]


def log_density(x, theta, dim=8, layers=6, hidden=128, bins=16, bf=True):
    """log q(x) of points x (n, dim)."""
    P = unpack(theta, dim, layers, hidden, bins)
    x = np.array(x, dtype=np.float64)
    logq = np.zeros(len(x))
    ml = masks(dim)
    for l in range(layers):
        A, B = ml[l % 6]
        raw = conditioner(x[:, A], P[l], bf).reshape(len(x), len(B), 3 * bins + 1)
        for jj, j in enumerate(B):
            y, ld = rqs_forward(x[:, j], raw[:, jj, :], bins)
            x[:, j] = y
            logq += ld
    return logq, x


def sample(z, theta, dim=8, layers=6, hidden=128, bins=16, bf=True):
    """x = T^{-1}(z) for z (n, dim) in [0,1); returns (x, log q(x))."""
    P = unpack(theta, dim, layers, hidden, bins)
    x = np.array(z, dtype=np.float64)
    ml = masks(dim)
    for l in reversed(range(layers)):
        A, B = ml[l % 6]
        raw = conditioner(x[:, A], P[l], bf).reshape(len(x), len(B), 3 * bins + 1)
        for jj, j in enumerate(B):
            x[:, j] = rqs_inverse(x[:, j], raw[:, jj, :], bins)
    logq, _ = log_density(x, theta, dim, layers, hidden, bins, bf)
    return x, logq


def loss(x, f, q0, theta, kind=1, **kw):
    """Training loss on weighted points (x_i, f_i = W_i / q0_i):
    kind 1: variance loss, mean(f^2 q0 / q_theta) / mean(f^2);
    kind 0: weighted maximum likelihood, -sum f log q_theta / sum f."""
    logq, _ = log_density(x, theta, **kw)
    if kind == 1:
        return np.mean(f * f * q0 * np.exp(-logq)) / np.mean(f * f)
    return -np.sum(f * logq) / np.sum(f)


def init_params(dim=8, layers=6, hidden=128, bins=16, seed=1):
    """Deterministic initial parameters: He-uniform W1, W2 (from a numpy generator
    seeded with `seed`), zero W3, b3 set so that every spline is the identity."""
    rng = np.random.default_rng(seed)
    P = []
    for _ in range(layers):
        for name, shape in layer_sizes(dim, hidden, bins):
            if name in ("W1", "W2"):
                lim = np.sqrt(6.0 / shape[0])
                P.append(rng.uniform(-lim, lim, size=shape).ravel())
            elif name == "b3":
                b = np.zeros(shape).reshape(dim // 2, 3 * bins + 1)
                b[:, 2 * bins:] = np.log(np.expm1(1.0 - MIN_D))
                P.append(b.ravel())
            else:
                P.append(np.zeros(int(np.prod(shape))))
    return np.concatenate(P)


# ---------------------------------------------------------------------------
# Analytic gradients (same chain of operations as the GPU backward kernel).

def _rqs_grad(x, raw, bins, gy, gl):
    """Given upstream gradients gy (of y) and gl (of log dy/dx), return the gradient
    with respect to x and to raw (n, 3K+1) of one rational-quadratic spline."""
    K = bins
    n = len(x)
    r = np.arange(n)
    wr, hr, dr = raw[:, :K], raw[:, K:2 * K], raw[:, 2 * K:]
    pw = np.exp(wr - wr.max(1, keepdims=True))
    pw /= pw.sum(1, keepdims=True)
    ph = np.exp(hr - hr.max(1, keepdims=True))
    ph /= ph.sum(1, keepdims=True)
    wid = MIN_W + (1 - K * MIN_W) * pw
    hei = MIN_H + (1 - K * MIN_H) * ph
    d = MIN_D + softplus(dr)
    X = np.concatenate([np.zeros((n, 1)), np.cumsum(wid, 1)], 1)
    Y = np.concatenate([np.zeros((n, 1)), np.cumsum(hei, 1)], 1)
    X[:, -1] = 1.0
    Y[:, -1] = 1.0
    k = np.clip(np.sum(X[:, 1:-1] <= x[:, None], 1), 0, K - 1)
    xk, w = X[r, k], X[r, k + 1] - X[r, k]
    hk = Y[r, k + 1] - Y[r, k]
    d0, d1 = d[r, k], d[r, k + 1]
    s = hk / w
    xi = (x - xk) / w
    om = xi * (1 - xi)
    den = s + (d0 + d1 - 2 * s) * om
    N1 = s * xi * xi + d0 * om
    Q = d1 * xi * xi + 2 * s * om + d0 * (1 - xi) ** 2
    # partials of y and L = log dy/dx in (xi, s, d0, d1) and explicit h
    dden = dict(xi=(d0 + d1 - 2 * s) * (1 - 2 * xi), s=1 - 2 * om, d0=om, d1=om)
    dN1 = dict(xi=2 * s * xi + d0 * (1 - 2 * xi), s=xi * xi, d0=om, d1=0.0)
    dQ = dict(xi=2 * d1 * xi + 2 * s * (1 - 2 * xi) - 2 * d0 * (1 - xi), s=2 * om,
              d0=(1 - xi) ** 2, d1=xi * xi)
    G = {}
    for v in ("xi", "s", "d0", "d1"):
        dy = hk * (dN1[v] * den - N1 * dden[v]) / (den * den)
        dL = dQ[v] / Q - 2 * dden[v] / den + (2 / s if v == "s" else 0.0)
        G[v] = gy * dy + gl * dL
    Gh = gy * N1 / den + G["s"] / w
    Gw = -G["xi"] * xi / w - G["s"] * s / w
    Gxk = -G["xi"] / w
    Gyk = gy
    gx = G["xi"] / w
    # knots: X[k] = sum_{i<k} wid_i, w = wid_k; likewise Y
    idx = np.arange(K)[None, :]
    gwid = Gxk[:, None] * (idx < k[:, None]) + Gw[:, None] * (idx == k[:, None])
    ghei = Gyk[:, None] * (idx < k[:, None]) + Gh[:, None] * (idx == k[:, None])
    gd = np.zeros((n, K + 1))
    gd[r, k] += G["d0"]
    gd[r, k + 1] += G["d1"]
    graw = np.zeros_like(raw)
    graw[:, :K] = (1 - K * MIN_W) * pw * (gwid - np.sum(pw * gwid, 1, keepdims=True))
    graw[:, K:2 * K] = (1 - K * MIN_H) * ph * (ghei - np.sum(ph * ghei, 1, keepdims=True))
    graw[:, 2 * K:] = gd / (1 + np.exp(-dr))
    return gx, graw


def loss_and_grad(x, coef, theta, kind=1, dim=8, layers=6, hidden=128, bins=16, bf=True):
    """Loss and gradient with respect to theta of the batch loss the GPU trains on.

    kind 1 (variance): L = mean_i coef_i * exp(-log q(x_i));
    kind 0 (weighted likelihood): L = -mean_i coef_i * log q(x_i).
    With bf=True the operands of the matrix products (activations, weights and the
    back-propagated gradients) are rounded to bfloat16 where the GPU rounds them."""
    q = bf16 if bf else (lambda v: v)
    n = len(x)
    P = unpack(theta, dim, layers, hidden, bins)
    ml = masks(dim)
    nB = dim // 2
    # forward, keeping each layer's input and activations
    cur = np.array(x, dtype=np.float64)
    saved = []
    logq = np.zeros(n)
    for l in range(layers):
        A, B = ml[l % 6]
        p = P[l]
        xa = cur[:, A]
        a1 = q(xa) @ q(p["W1"]) + p["b1"]
        h1 = np.maximum(a1, 0.0)
        a2 = q(h1) @ q(p["W2"]) + p["b2"]
        h2 = np.maximum(a2, 0.0)
        raw = (q(h2) @ q(p["W3"]) + p["b3"]).reshape(n, nB, 3 * bins + 1)
        saved.append((cur.copy(), xa, h1, h2, raw))
        for jj, j in enumerate(B):
            y, ld = rqs_forward(cur[:, j], raw[:, jj, :], bins)
            cur[:, j] = y
            logq += ld
    if kind == 1:
        e = coef * np.exp(-logq)
        L = np.mean(e)
        gld = -e / n
    else:
        L = -np.mean(coef * logq)
        gld = -coef / n
    grads = []
    gcur = np.zeros((n, dim))  # dL/d(output of the layer being processed)
    for l in reversed(range(layers)):
        A, B = ml[l % 6]
        p = P[l]
        xin, xa, h1, h2, raw = saved[l]
        graw = np.zeros((n, nB, 3 * bins + 1))
        gin = gcur.copy()
        for jj, j in enumerate(B):
            gx, gr = _rqs_grad(xin[:, j], raw[:, jj, :], bins, gcur[:, j], gld)
            gin[:, j] = gx
            graw[:, jj, :] = gr
        graw = graw.reshape(n, -1)
        gW3 = q(h2).T @ q(graw)
        gb3 = graw.sum(0)
        gh2 = (q(graw) @ q(p["W3"]).T) * (h2 > 0)
        gW2 = q(h1).T @ q(gh2)
        gb2 = gh2.sum(0)
        gh1 = (q(gh2) @ q(p["W2"]).T) * (h1 > 0)
        gW1 = q(xa).T @ q(gh1)
        gb1 = gh1.sum(0)
        gxa = q(gh1) @ q(p["W1"]).T
        gin[:, A] += gxa
        gcur = gin
        grads.append(dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, W3=gW3, b3=gb3))
    grads = grads[::-1]
    flat = []
    for l in range(layers):
        for name, shape in layer_sizes(dim, hidden, bins):
            flat.append(np.asarray(grads[l][name]).ravel())
    return L, np.concatenate(flat), logq


def adam_step(theta, grad, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015) with bias correction; t counts from 1."""
    m[:] = beta1 * m + (1 - beta1) * grad
    v[:] = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    theta -= lr * mh / (np.sqrt(vh) + eps)
    return theta
