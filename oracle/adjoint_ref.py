"""FP64 host reference of the differentiable forward and its gradient —
TEST INFRASTRUCTURE ONLY (the checker of n2m_meshify_backward).

For a fixed topology (the vertex sources reported by the oracle's Lewiner
marching cubes), the forward maps the input volume to vertex positions in
float64 without any float rounding:
  s = S img                  separable 5-tap blur, faces left unfiltered
                             (src/meshify.c:170-216, here in exact float64)
  edge vertex on (p, q):     x = p + u e_axis, u = (s_p - iso) / (s_p - s_q)
                             (src/MarchingCubes.c:935-1026)
  c-vertex:                  mean of the cube's crossing edge vertices
                             (src/MarchingCubes.c:1029-1082)
  HC smoothing, K iters:     the oracle's laplacian_smoothHC (src/quadric.c:343-394)
and `gradient` is the analytic adjoint of the same map (sparse matrices).
"""
import numpy as np
import scipy.sparse as sp

TAPS = (0.05, 0.225, 0.45, 0.225, 0.05)
FLT_EPS = 1.19209290e-07
# cube edge e: owner corner, axis, corner a, corner b (edge numbering of the tables)
EDGES = ((0, 0, 0, 1), (1, 1, 1, 2), (3, 0, 3, 2), (0, 1, 0, 3), (4, 0, 4, 5), (5, 1, 5, 6), (7, 0, 7, 6), (4, 1, 4, 7),
         (0, 2, 0, 4), (1, 2, 1, 5), (2, 2, 2, 6), (3, 2, 3, 7))
CORNER = [((p ^ (p >> 1)) & 1, (p >> 1) & 1, (p >> 2) & 1) for p in range(8)]


def _pass(a, axis, transpose=False):
    n = a.shape[axis]
    if n < 5:
        return a.copy()
    out = a.copy()
    idx = [slice(None)] * 3
    if not transpose:
        idx[axis] = slice(2, n - 2)
        acc = 0
        for k, w in enumerate(TAPS):
            sl = [slice(None)] * 3
            sl[axis] = slice(k, n - 4 + k)
            acc = acc + w * a[tuple(sl)]
        out[tuple(idx)] = acc
        return out
    # transpose: boundary rows pass through, interior rows scatter their taps
    res = np.zeros_like(a)
    for rows in (slice(0, 2), slice(n - 2, n)):
        sl = [slice(None)] * 3
        sl[axis] = rows
        res[tuple(sl)] += a[tuple(sl)]
    src = [slice(None)] * 3
    src[axis] = slice(2, n - 2)
    for k, w in enumerate(TAPS):
        dst = [slice(None)] * 3
        dst[axis] = slice(k, n - 4 + k)
        res[tuple(dst)] += w * a[tuple(src)]
    return res


def smooth64(img):
    a = np.asarray(img, np.float64)
    if min(a.shape) < 5:
        return a.copy()
    for axis in (2, 1, 0):                 # x pass, y pass, z pass
        a = _pass(a, axis)
    return a


def smooth64_T(g):
    a = np.asarray(g, np.float64)
    if min(a.shape) < 5:
        return a.copy()
    for axis in (0, 1, 2):
        a = _pass(a, axis, transpose=True)
    return a


class Topology:
    """Vertex sources over the padded box: (kind, grid index, axis) per vertex."""

    def __init__(self, src, lo, hi, shape):
        self.src = np.asarray(src)
        self.lo = np.asarray(lo)
        self.n = np.asarray(hi) - np.asarray(lo) + 1
        self.shape = shape   # (nz, ny, nx)
        nz, ny, nx = shape
        NX, NY = self.n[0], self.n[1]
        g = self.src[:, 1]
        self.gp = np.stack([g % NX, (g // NX) % NY, g // (NX * NY)], 1) + self.lo   # voxel (x,y,z)
        if (self.gp.max(0) + 1 >= [nx, ny, nz]).any() or (self.gp.min(0) < 1).any():
            raise ValueError("topology touches the volume boundary; pick an interior test volume")

    def _val(self, s, xyz):
        return s[xyz[..., 2], xyz[..., 1], xyz[..., 0]]

    def _edges(self, s, iso):
        """vectorised edge vertices: positions and the pieces of their adjoint"""
        e = self.src[:, 0] == 0
        p = self.gp[e]
        ax = self.src[e, 2]
        q = p + np.eye(3, dtype=p.dtype)[ax]
        c0 = self._val(s, p) - iso
        c1 = self._val(s, q) - iso
        c0 = np.where(np.abs(c0) < FLT_EPS, FLT_EPS, c0)
        c1 = np.where(np.abs(c1) < FLT_EPS, FLT_EPS, c1)
        x = p.astype(np.float64)
        x[np.arange(len(p)), ax] += c0 / (c0 - c1)
        return e, p, q, ax, c0, c1, x

    def positions(self, s, iso):
        P = np.zeros((len(self.src), 3))
        e, _, _, _, _, _, x = self._edges(s, iso)
        P[e] = x
        for i in np.nonzero(~e)[0]:
            p = self.gp[i]
            pts = [self._edge_pos(s, iso, p + CORNER[own], ax)[0] for own, ax, a, b in EDGES
                   if self._cross(s, iso, p, a, b)]
            P[i] = np.mean(pts, 0)
        return P

    def _cval(self, s, iso, xyz):
        c = self._val(s, np.asarray(xyz)) - iso
        return FLT_EPS if abs(c) < FLT_EPS else c

    def _cross(self, s, iso, p, a, b):
        return (self._cval(s, iso, p + CORNER[a]) > 0) != (self._cval(s, iso, p + CORNER[b]) > 0)

    def _edge_pos(self, s, iso, p, axis):
        q = p.copy()
        q[axis] += 1
        c0, c1 = self._cval(s, iso, p), self._cval(s, iso, q)
        u = c0 / (c0 - c1)
        x = p.astype(np.float64).copy()
        x[axis] += u
        return x, p, q, c0, c1

    def adjoint(self, s, iso, gP):
        """dL/ds from dL/dpositions (float64 volume)"""
        gs = np.zeros(self.shape)
        e, p, q, ax, c0, c1, _ = self._edges(s, iso)
        g = gP[e][np.arange(len(p)), ax]
        den = c0 - c1
        np.add.at(gs, (p[:, 2], p[:, 1], p[:, 0]), g * (-c1 / den ** 2))
        np.add.at(gs, (q[:, 2], q[:, 1], q[:, 0]), g * (c0 / den ** 2))
        for i in np.nonzero(~e)[0]:
            pc = self.gp[i]
            edges = [(own, a2) for own, a2, a, b in EDGES if self._cross(s, iso, pc, a, b)]
            for own, a2 in edges:
                _, pp, qq, d0, d1 = self._edge_pos(s, iso, pc + CORNER[own], a2)
                dd = d0 - d1
                gs[pp[2], pp[1], pp[0]] += gP[i, a2] / len(edges) * (-d1 / dd ** 2)
                gs[qq[2], qq[1], qq[0]] += gP[i, a2] / len(edges) * (d0 / dd ** 2)
        return gs


def laplacian_matrix(tris, n):
    t = np.asarray(tris, np.int64)
    rows = np.concatenate([t[:, 0], t[:, 0], t[:, 1], t[:, 1], t[:, 2], t[:, 2]])
    cols = np.concatenate([t[:, 1], t[:, 2], t[:, 0], t[:, 2], t[:, 0], t[:, 1]])
    W = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))
    num = np.asarray(W.sum(1)).ravel()
    inv = np.where(num > 0, 1.0 / np.maximum(num, 1), 0.0)
    L = sp.diags(inv) @ W + sp.diags((num == 0).astype(np.float64))
    return L.tocsr()


def hc_adjoint(tris, n, g, alpha, beta, iters, border):
    L = laplacian_matrix(tris, n)
    I = sp.identity(n, format="csr")
    A = beta * (1 - alpha) * I + (1 - beta) * (2 - alpha) * L - (1 - beta) * (L @ L)
    B = alpha * beta * I + alpha * (1 - beta) * L
    mask = (~border).astype(np.float64)[:, None]
    lam = mask * g
    go = (1 - mask) * g
    At, Bt = A.T.tocsr(), B.T.tocsr()
    for _ in range(iters):
        go = go + Bt @ lam
        lam = At @ lam
    return go + lam


def loss_and_grad(P, center, radius):
    d = P - np.asarray(center)
    r = np.linalg.norm(d, axis=1)
    loss = np.sum((r - radius) ** 2)
    g = (2 * (r - radius) / r)[:, None] * d
    return loss, g


class Problem:
    """FP64 forward/gradient of L(img) = sum(|v - c| - R)^2 over the vertices of
    meshify(img, iso, -p 1 -l 0 -b 0, Lewiner) followed by `iters` HC
    iterations (alpha 0.1, beta 0.5, border locked), topology frozen at img."""

    def __init__(self, oracle, img, iso, iters, center, radius):
        img = np.asarray(img, np.float32)
        self.img, self.iso, self.iters, self.center, self.radius = img, float(iso), iters, center, radius
        prep = oracle.prepare_volume(img, iso, True, False, False)
        vol, self.iso_used, lo, hi, _ = prep
        t, p, src = oracle.marching_cubes_sources(vol, lo, hi, self.iso_used)
        mesh = oracle.meshify(img, iso, 0, True, False, False)
        if len(mesh[1]) != len(p):
            raise ValueError("the weld merged vertices; pick another test volume")
        self.tris = mesh[0]
        self.topo = Topology(src, lo, hi, img.shape)
        self.oracle = oracle
        self.border = oracle.border_vertices(self.tris, len(p))

    def positions(self, img):
        return self.topo.positions(smooth64(img), self.iso_used)

    def smoothed_positions(self, img):
        P = self.positions(img)
        if self.iters:
            P = self.oracle.laplacian_smoothHC(P, self.tris, 0.1, 0.5, self.iters, True)
        return P

    def loss(self, img):
        return loss_and_grad(self.smoothed_positions(img), self.center, self.radius)[0]

    def gradient(self, img):
        s = smooth64(img)
        P = self.topo.positions(s, self.iso_used)
        Ps = self.oracle.laplacian_smoothHC(P, self.tris, 0.1, 0.5, self.iters, True) if self.iters else P
        _, g = loss_and_grad(Ps, self.center, self.radius)
        if self.iters:
            g = hc_adjoint(self.tris, len(P), g, 0.1, 0.5, self.iters, self.border)
        return smooth64_T(self.topo.adjoint(s, self.iso_used, g))

    def central_difference(self, img, voxels, h):
        out = []
        base = np.asarray(img, np.float64)
        for z, y, x in voxels:
            a, b = base.copy(), base.copy()
            a[z, y, x] += h
            b[z, y, x] -= h
            out.append((self.loss(a) - self.loss(b)) / (2 * h))
        return np.array(out)
