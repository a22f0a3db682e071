"""CPU oracle of the learned proposal's encoder, loss and gradients (NumPy, Float64).

TEST INFRASTRUCTURE ONLY: tests/ use it to check the library's hand-written CUDA forward and
backward kernels (imagequilting.jl_gb300/csrc/iq_proposal.cu); the product never imports it.

The proposal has no counterpart in the reference (ImageQuilting.jl scans every training-image
position, src/iqsim.jl:206 and src/utils.jl:5-13). Its encoder maps the masked overlap region
of a tile, or a training-image window under the same mask, to a 64-d vector:

  cells    the tile is split into a grid G = (min(tx, 8), min(ty, 8), min(tz, 4)) of cells of
           c_d = ceil(t_d / G_d) voxels; per cell three inputs: the mask fraction, and the sums
           of the values and of their squares over the cell's masked voxels, each divided by
           the cell volume
  layer 1  1x1x1 convolution 3 -> 32 channels, bias, ReLU            (per cell)
  layer 2  3x3x3 convolution 32 -> 32, stride 2, zero padding 1, bias, ReLU
  layer 3  3x3x3 convolution 32 -> 32, stride 2, zero padding 1, bias, ReLU
  output   linear (32 x cells of layer 3) -> 64, bias

The loss of one anchor (a template) with its positive window (one of its exact candidates) and
negative windows (random positions) is InfoNCE on squared distances:
  z_j = -|e_a - e_j|^2 / T,   L = -z_pos + log sum_j exp(z_j).
Arrays are column-major over the cell grid (x fastest), channels outermost.
"""
import math

import numpy as np

CH = 32
EMB = 64
NIN = 3


def grid_dims(tile):
    t = tuple(int(v) for v in tile) + (1,) * (3 - len(tile))
    G = (min(t[0], 8), min(t[1], 8), min(t[2], 4))
    c = tuple(math.ceil(ti / gi) for ti, gi in zip(t, G))
    return G, c


def down(G):
    return tuple((g + 1) // 2 for g in G)


def param_shapes(tile):
    G, _ = grid_dims(tile)
    G3 = down(down(G))
    return {"w1": (CH, NIN), "b1": (CH,), "w2": (CH, CH, 27), "b2": (CH,),
            "w3": (CH, CH, 27), "b3": (CH,), "w4": (EMB, CH * int(np.prod(G3))), "b4": (EMB,)}


def init_params(tile, seed):
    """He-style initialization with the Philox-free NumPy generator (tests only)."""
    rng = np.random.default_rng(seed)
    p = {}
    for k, s in param_shapes(tile).items():
        if k.startswith("b"):
            p[k] = np.zeros(s)
        else:
            fan_in = int(np.prod(s[1:]))
            p[k] = rng.normal(size=s) * math.sqrt(2.0 / fan_in)
    return p


def cell_features(values, mask, tile):
    """(3, G) inputs of one window: mask fraction, masked sum / volume, masked sum of squares /
    volume. values, mask: arrays of the tile's shape."""
    G, c = grid_dims(tile)
    t = tuple(int(v) for v in tile) + (1,) * (3 - len(tile))
    v = np.zeros(t)
    m = np.zeros(t)
    v[tuple(slice(0, s) for s in np.shape(values))] = np.asarray(values, np.float64).reshape(
        np.shape(values))
    m[tuple(slice(0, s) for s in np.shape(mask))] = np.asarray(mask, np.float64)
    v = v.reshape(t)
    m = m.reshape(t)
    vol = float(c[0] * c[1] * c[2])
    X = np.zeros((NIN,) + G)
    for i in range(G[0]):
        for j in range(G[1]):
            for k in range(G[2]):
                sl = (slice(i * c[0], (i + 1) * c[0]), slice(j * c[1], (j + 1) * c[1]),
                      slice(k * c[2], (k + 1) * c[2]))
                mm = m[sl]
                vv = v[sl] * mm
                X[0, i, j, k] = mm.sum() / vol
                X[1, i, j, k] = vv.sum() / vol
                X[2, i, j, k] = (vv * v[sl]).sum() / vol
    return X


def _taps():
    """(t, dx, dy, dz) with t = dx + 3 dy + 9 dz (column-major), offsets -1..1."""
    return [(dx + 3 * dy + 9 * dz, dx - 1, dy - 1, dz - 1)
            for dz in range(3) for dy in range(3) for dx in range(3)]


def conv_s2(h, w, b):
    G = h.shape[1:]
    Go = down(G)
    out = np.zeros((w.shape[0],) + Go)
    for o in np.ndindex(*Go):
        acc = b.astype(np.float64).copy()
        for t, dx, dy, dz in _taps():
            x, y, z = 2 * o[0] + dx, 2 * o[1] + dy, 2 * o[2] + dz
            if 0 <= x < G[0] and 0 <= y < G[1] and 0 <= z < G[2]:
                acc += w[:, :, t] @ h[:, x, y, z]
        out[(slice(None),) + o] = acc
    return out


def conv_s2_backward(h, w, gout):
    """Gradients of conv_s2 w.r.t. its input h and its weights w, given d/d(out)."""
    G = h.shape[1:]
    Go = down(G)
    gh = np.zeros_like(h)
    gw = np.zeros_like(w)
    for o in np.ndindex(*Go):
        go = gout[(slice(None),) + o]
        for t, dx, dy, dz in _taps():
            x, y, z = 2 * o[0] + dx, 2 * o[1] + dy, 2 * o[2] + dz
            if 0 <= x < G[0] and 0 <= y < G[1] and 0 <= z < G[2]:
                gw[:, :, t] += np.outer(go, h[:, x, y, z])
                gh[:, x, y, z] += w[:, :, t].T @ go
    return gh, gw, gout.sum(axis=tuple(range(1, gout.ndim)))


def forward(p, X):
    """Embedding of one window and the activations the backward pass needs."""
    z1 = np.einsum("ci,ixyz->cxyz", p["w1"], X) + p["b1"][:, None, None, None]
    h1 = np.maximum(z1, 0)
    z2 = conv_s2(h1, p["w2"], p["b2"])
    h2 = np.maximum(z2, 0)
    z3 = conv_s2(h2, p["w3"], p["b3"])
    h3 = np.maximum(z3, 0)
    f = h3.reshape(h3.shape[0], -1, order="F").reshape(-1, order="F")  # cell-major, channel fastest
    e = p["w4"] @ f + p["b4"]
    return e, (X, z1, h1, z2, h2, z3, h3, f)


def backward(p, cache, ge):
    """Parameter gradients of one window given d/d(embedding)."""
    X, z1, h1, z2, h2, z3, h3, f = cache
    g = {}
    g["w4"] = np.outer(ge, f)
    g["b4"] = ge.copy()
    gf = p["w4"].T @ ge
    gh3 = gf.reshape(h3.shape[0], -1, order="F").reshape(h3.shape, order="F")
    gz3 = gh3 * (z3 > 0)
    gh2, g["w3"], g["b3"] = conv_s2_backward(h2, p["w3"], gz3)
    gz2 = gh2 * (z2 > 0)
    gh1, g["w2"], g["b2"] = conv_s2_backward(h1, p["w2"], gz2)
    gz1 = gh1 * (z1 > 0)
    g["w1"] = np.einsum("cxyz,ixyz->ci", gz1, X)
    g["b1"] = gz1.sum(axis=(1, 2, 3))
    return g


def infonce(ea, ep, en, temp):
    """Loss of one anchor and d/d of the anchor, positive and negative embeddings."""
    E = np.vstack([ep[None], en])
    d = ea[None] - E
    z = -np.sum(d * d, axis=1) / temp
    zmax = z.max()
    ex = np.exp(z - zmax)
    s = ex.sum()
    loss = -z[0] + zmax + math.log(s)
    gz = ex / s
    gz[0] -= 1.0
    # z_j = -|ea - E_j|^2 / T: dz/dea = -2 (ea - E_j) / T, dz/dE_j = 2 (ea - E_j) / T
    gea = np.sum(gz[:, None] * (-2.0 * d / temp), axis=0)
    gE = gz[:, None] * (2.0 * d / temp)
    return loss, gea, gE[0], gE[1:]


def batch_loss_and_grads(p, anchors, positives, negatives, temp):
    """Mean InfoNCE over a batch: anchors (B, 3, G), positives (B, 3, G), negatives
    (B, Nn, 3, G). Returns (loss, parameter gradients)."""
    B = len(anchors)
    grads = {k: np.zeros_like(v) for k, v in p.items()}
    total = 0.0
    for b in range(B):
        ea, ca = forward(p, anchors[b])
        ep, cp = forward(p, positives[b])
        outs = [forward(p, x) for x in negatives[b]]
        en = np.array([o[0] for o in outs])
        loss, gea, gep, gen = infonce(ea, ep, en, temp)
        total += loss / B
        for ge, c in [(gea, ca), (gep, cp)] + [(gen[i], outs[i][1]) for i in range(len(outs))]:
            g = backward(p, c, ge / B)
            for k in grads:
                grads[k] += g[k]
    return total, grads
