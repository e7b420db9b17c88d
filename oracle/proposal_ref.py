"""NumPy restatement of the learned crossing proposal (features, network, loss,
gradients, Adam).  TEST INFRASTRUCTURE ONLY: the proposal tests check the CUDA
kernels of gpis_extend_gb300/csrc/proposal.cu against it.

The network (the proposal model of the flight benchmark's learned path):
  history x_j = (mean_j, slope_j), j = 0..7: the mean SDF and its slope along the
  ray at the centres of eight equal parts of [near, far];
  globals g (8): t_max, local length scale, conditioned value and derivative,
  first-scatter flag, amplitude, step / t_max, mean at near;
  GRU, hidden 32 (PyTorch gate order r, z, n) over the eight history steps;
  MLP [h_8, g] (40, padded to 48) -> 64 -> 64 -> 64 (GELU, tanh form) -> 25;
  outputs: 8 mixture logits, 8 locations (sigmoid), 8 scales (softplus + 1e-3)
  of a logistic mixture over u = (t - near) / (far - near), and a miss logit.
Loss per flight: hit  -log(1 - q) - log sum_k pi_k Logistic(u*; m_k, s_k)
                 miss -log q,  q = sigmoid(miss logit).
Every GEMM takes BF16 inputs (round to nearest even) and accumulates in FP32;
this restatement rounds the same operands and accumulates in FP64.
"""
import numpy as np

HID = 32
N_IN = 16          # GRU input, padded from 2
MLP_IN = 48        # [h (32), globals (8), zeros (8)]
WIDTH = 64
N_OUT = 32         # 25 used
N_COMP = 8
N_HIST = 8
N_FEAT = 24

# parameter tensors in the order of the flat parameter vector: (name, shape (out, in))
PARAMS = [("w_ih", (3 * HID, N_IN)), ("b_ih", (3 * HID,)), ("w_hh", (3 * HID, HID)), ("b_hh", (3 * HID,)),
          ("w1", (WIDTH, MLP_IN)), ("b1", (WIDTH,)), ("w2", (WIDTH, WIDTH)), ("b2", (WIDTH,)),
          ("w3", (WIDTH, WIDTH)), ("b3", (WIDTH,)), ("w4", (N_OUT, WIDTH)), ("b4", (N_OUT,))]


def n_params():
    return sum(int(np.prod(s)) for _, s in PARAMS)


def unflatten(flat):
    out, o = {}, 0
    for name, shape in PARAMS:
        k = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + k], np.float64).reshape(shape)
        o += k
    return out


def flatten(p):
    return np.concatenate([np.asarray(p[name], np.float64).ravel() for name, _ in PARAMS])


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(np.isnan(a), u, r)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def mm(x, w):
    """x @ w.T with BF16 operands, accumulated in float64 (the kernels accumulate in FP32)."""
    return bf16(x) @ bf16(w).T


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def softplus(x):
    return np.logaddexp(0.0, x)


GELU_C = np.sqrt(2.0 / np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    u = GELU_C * (x + 0.044715 * x ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3 * 0.044715 * x * x)


def forward(p, feats):
    """Returns (outputs (n, 32), cache for backward)."""
    f = np.asarray(feats, np.float64)
    n = f.shape[0]
    h = np.zeros((n, HID))
    cache = {"h": [h], "x": [], "r": [], "z": [], "nn": [], "ghn": []}
    for j in range(N_HIST):
        x = np.zeros((n, N_IN))
        x[:, 0:2] = f[:, 2 * j:2 * j + 2]
        gi = mm(x, p["w_ih"]) + p["b_ih"]
        gh = mm(h, p["w_hh"]) + p["b_hh"]
        r = sigmoid(gi[:, :HID] + gh[:, :HID])
        z = sigmoid(gi[:, HID:2 * HID] + gh[:, HID:2 * HID])
        nn = np.tanh(gi[:, 2 * HID:] + r * gh[:, 2 * HID:])
        h = (1.0 - z) * nn + z * h
        cache["x"].append(x)
        cache["r"].append(r)
        cache["z"].append(z)
        cache["nn"].append(nn)
        cache["ghn"].append(gh[:, 2 * HID:])
        cache["h"].append(h)
    u = np.zeros((n, MLP_IN))
    u[:, :HID] = h
    u[:, HID:HID + 8] = f[:, 16:24]
    a1 = mm(u, p["w1"]) + p["b1"]
    y1 = gelu(a1)
    a2 = mm(y1, p["w2"]) + p["b2"]
    y2 = gelu(a2)
    a3 = mm(y2, p["w3"]) + p["b3"]
    y3 = gelu(a3)
    o = mm(y3, p["w4"]) + p["b4"]
    cache.update(u=u, a1=a1, y1=y1, a2=a2, y2=y2, a3=a3, y3=y3)
    return o, cache


def mixture(o):
    logits = o[:, 0:8]
    m = sigmoid(o[:, 8:16])
    s = softplus(o[:, 16:24]) + 1e-3
    return logits, m, s, o[:, 24]


def loss_and_grad_out(o, u_star, hit):
    """Mean NLL over the batch and its gradient w.r.t. the 32 outputs."""
    n = o.shape[0]
    logits, m, s, ql = mixture(o)
    lse_pi = np.logaddexp.reduce(logits, axis=1)
    logpi = logits - lse_pi[:, None]
    y = (u_star[:, None] - m) / s
    logf = -softplus(-y) - softplus(y) - np.log(s)
    comp = logpi + logf
    lse = np.logaddexp.reduce(comp, axis=1)
    hitf = hit.astype(np.float64)
    nll = hitf * (softplus(ql) - lse) + (1.0 - hitf) * softplus(-ql)
    g = np.zeros_like(o)
    w = np.exp(comp - lse[:, None])                 # responsibilities
    g[:, 0:8] = hitf[:, None] * (np.exp(logpi) - w)
    # d(-logf)/dy = sigmoid(y) - sigmoid(-y) = tanh(y / 2); dy/dm = -1/s; dy/ds = -y/s
    dldy = np.tanh(y / 2.0)
    dm = hitf[:, None] * w * dldy * (-1.0 / s)
    ds = hitf[:, None] * w * (dldy * (-y / s) + 1.0 / s)
    g[:, 8:16] = dm * m * (1.0 - m)
    g[:, 16:24] = ds * sigmoid(o[:, 16:24])
    g[:, 24] = hitf * sigmoid(ql) - (1.0 - hitf) * sigmoid(-ql)
    return float(nll.mean()), g / n


def backward(p, cache, g_out):
    """Gradients of every parameter given dL/d(outputs); BF16 operands as the kernels."""
    gr = {k: np.zeros_like(v) for k, v in p.items()}
    da = g_out
    gr["w4"] = bf16(da).T @ bf16(cache["y3"])
    gr["b4"] = da.sum(0)
    dy = bf16(da) @ bf16(p["w4"])
    for k, a, x in (("3", cache["a3"], cache["y2"]), ("2", cache["a2"], cache["y1"]), ("1", cache["a1"], cache["u"])):
        da = dy * gelu_grad(a)
        gr["w" + k] = bf16(da).T @ bf16(x)
        gr["b" + k] = da.sum(0)
        dy = bf16(da) @ bf16(p["w" + k])
    dh = dy[:, :HID]
    for j in reversed(range(N_HIST)):
        h_prev = cache["h"][j]
        r, z, nn, ghn, x = cache["r"][j], cache["z"][j], cache["nn"][j], cache["ghn"][j], cache["x"][j]
        dz = dh * (h_prev - nn) * z * (1.0 - z)
        dn = dh * (1.0 - z) * (1.0 - nn * nn)
        dr = dn * ghn * r * (1.0 - r)
        dgi = np.concatenate([dr, dz, dn], axis=1)
        dgh = np.concatenate([dr, dz, dn * r], axis=1)
        gr["w_ih"] += bf16(dgi).T @ bf16(x)
        gr["b_ih"] += dgi.sum(0)
        gr["w_hh"] += bf16(dgh).T @ bf16(h_prev)
        gr["b_hh"] += dgh.sum(0)
        dh = dh * z + bf16(dgh) @ bf16(p["w_hh"])
    return gr


def adam(flat, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v


def interval(o, far_frac=3.0):
    """The proposal: the dominant component's [m - c s, m + c s] in u, clipped to [0, 1],
    and the miss probability."""
    logits, m, s, ql = mixture(o)
    k = np.argmax(logits, axis=1)
    mk = m[np.arange(len(k)), k]
    sk = s[np.arange(len(k)), k]
    return np.clip(mk - far_frac * sk, 0, 1), np.clip(mk + far_frac * sk, 0, 1), sigmoid(ql)


def _mean_and_grad(desc, p):
    """Mean SDF and its gradient (sphere, plane, torus, torus union plane), float64."""
    q = np.array(desc.mean_params[:8], np.float64)
    kind = int(desc.mean_kind)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    if kind == 0:
        d = p - q[:3]
        r = np.linalg.norm(d, axis=1)
        return r - q[3], d / r[:, None]
    if kind == 3:
        return p @ q[:3] - q[3], np.broadcast_to(q[:3], p.shape)
    if kind in (4, 5):
        px, py, pz = x - q[0], y - q[1], z - q[2]
        rxz = np.sqrt(px * px + pz * pz)
        s = rxz - q[3]
        ln = np.sqrt(s * s + py * py)
        mean = ln - q[4]
        g = np.stack([np.where(rxz > 0, s / ln * px / np.maximum(rxz, 1e-30), 0.0), py / ln,
                      np.where(rxz > 0, s / ln * pz / np.maximum(rxz, 1e-30), 0.0)], axis=1)
        if kind == 5:
            pl = y - q[5]
            use = pl < mean
            mean = np.where(use, pl, mean)
            g = np.where(use[:, None], np.array([0.0, 1.0, 0.0]), g)
        return mean, g
    raise ValueError("mean kind without a restated gradient")


def features(desc, origin_near, dir_far, seeds, prev):
    """The 24 features of gpis_proposal_features (float64)."""
    o = np.asarray(origin_near, np.float64)
    d = np.asarray(dir_far, np.float64)
    n = len(o)
    near, far = o[:, 3], d[:, 3]
    tm = np.maximum(far - near, 0.0)
    f = np.zeros((n, N_FEAT))
    for j in range(N_HIST):
        t = near + (j + 0.5) * 0.125 * tm
        p = o[:, :3] + t[:, None] * d[:, :3]
        mv, g = _mean_and_grad(desc, p)
        f[:, 2 * j] = np.clip(mv, -4, 4)
        f[:, 2 * j + 1] = np.clip(np.sum(g * d[:, :3], axis=1), -4, 4)
    q = desc.ls_params
    varying = desc.ls_kind != 0
    ls = q[0] + q[1] * np.sin(q[2] * o[:, 0]) * np.cos(q[3] * o[:, 2]) if varying else np.ones(n)
    ell = ls * desc.length_scale * desc.aniso[0]
    first = (np.asarray(seeds)[:, 2] & 1) != 0
    pv = np.asarray(prev, np.float64)
    amp = sum(desc.octave_sigma[:desc.n_octaves]) if desc.n_octaves > 1 else desc.sigma
    step = np.minimum(tm / desc.min_step, desc.step_size)
    f[:, 16] = tm * 0.25
    f[:, 17] = 10 * ell
    f[:, 18] = np.where(first, 0.0, np.clip(pv[:, 0], -4, 4))
    f[:, 19] = np.where(first, 0.0, np.clip(np.sum(pv[:, 1:] * d[:, :3], axis=1), -4, 4))
    f[:, 20] = first.astype(np.float64)
    f[:, 21] = 10 * amp
    f[:, 22] = np.where(tm > 0, np.minimum(step / np.where(tm > 0, tm, 1), 1.0), 1.0)
    m0, _ = _mean_and_grad(desc, o[:, :3] + near[:, None] * d[:, :3])
    f[:, 23] = np.clip(m0, -4, 4)
    return f
