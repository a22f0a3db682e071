"""Cut costs with the reference's unquantized Float64 capacities (src/graphcut.jl:29-48).

The oracle and the library round every capacity to a multiple of 2^(ilogb(cmax) - 47) so that
their max-flows are exact; these helpers evaluate a cut mask with the capacities as the
reference computes them (Float32 differences and gradient sums, Float64 division by
sum + eps()) and give the unquantized maximum-flow value, so a test can show that the mask is a
minimum cut of the unquantized graph too (equal cost to rounding)."""
import numpy as np

EPS = 2.220446049250313e-16


def edges(A, B):
    """(u, v, capacity) of every lattice edge, u < v, in column-major order per dimension."""
    A = np.asarray(A, np.float32)
    B = np.asarray(B, np.float32)
    shape = A.shape
    n = A.size
    a = A.ravel(order="F")
    b = B.ravel(order="F")
    idx = np.arange(n).reshape(shape, order="F")
    out = []
    for d in range(A.ndim):
        if shape[d] < 2:
            continue
        for u in np.ndindex(*shape):
            if u[d] + 1 >= shape[d]:
                continue
            v = tuple(x + (1 if i == d else 0) for i, x in enumerate(u))
            w = tuple(x + (2 if i == d else 0) for i, x in enumerate(u))
            iu, iv = idx[u], idx[v]
            du = np.float32(abs(a[iu] - b[iu]))
            dv = np.float32(abs(a[iv] - b[iv]))
            gau = np.float32(abs(a[iv] - a[iu]))
            gbu = np.float32(abs(b[iv] - b[iu]))
            if u[d] + 2 < shape[d]:
                iw = idx[w]
                gav = np.float32(abs(a[iw] - a[iv]))
                gbv = np.float32(abs(b[iw] - b[iv]))
            else:
                gav, gbv = gau, gbu
            num = np.float32(du + dv)
            den = np.float32(np.float32(np.float32(gau + gav) + gbu) + gbv)
            out.append((int(iu), int(iv), float(num) / (float(den) + EPS)))
    return out


def cut_cost(A, B, mask):
    m = np.asarray(mask, bool).ravel(order="F")
    return sum(c for u, v, c in edges(A, B) if m[u] != m[v])


def maxflow_value(A, B, dim):
    """Maximum s-t flow of the unquantized graph (s -> first slice, last slice -> t)."""
    import networkx as nx
    shape = np.shape(A)
    G = nx.DiGraph()
    for u, v, c in edges(A, B):
        G.add_edge(u, v, capacity=c)
        G.add_edge(v, u, capacity=c)
    idx = np.arange(int(np.prod(shape))).reshape(shape, order="F")
    for u in np.take(idx, 0, axis=dim).ravel():
        G.add_edge("s", int(u))
    for v in np.take(idx, shape[dim] - 1, axis=dim).ravel():
        G.add_edge(int(v), "t")
    return nx.maximum_flow_value(G, "s", "t", flow_func=nx.algorithms.flow.preflow_push)
