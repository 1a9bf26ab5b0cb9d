"""Oracle of f2disp (test infrastructure only): the reference's nodal least-squares fit of
positions to the deformation gradient (src/f2disp.f:16-135, form_BTB :136-400) restated
with numpy/scipy: the hexahedral mesh of blkgen (src/oumodel.f:178-330; nodes x fastest,
elements z fastest, node numbering of vblke :612-700), trilinear shape functions,
B^T B integrated with 2x2x2 Gauss points, B^T F with one point at the element centre,
node 1 held at the origin, the sparse system solved directly (PARDISO's role), and
u = x - X."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# local node signs of the 8-node hexahedron (vblke's nd table order)
_SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                   [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)


def element_grad(xi, h):
    """Exact: N_a = prod_d (1 + s_d xi_d)/2; dN_a/dX_d = (s_d / h_d) prod_{e != d} (1 + s_e xi_e)/2."""
    g = np.empty((8, 3))
    for a, s in enumerate(_SIGNS):
        f = [(1 + s[d] * xi[d]) / 2 for d in range(3)]
        for d in range(3):
            o = [e for e in range(3) if e != d]
            g[a, d] = s[d] / h[d] * f[o[0]] * f[o[1]]
    return g


def displacements(F, N, lengths):
    """F: (9, N^3) with voxel v = a + N b + N^2 c (a along Z, c along X).  Returns u as the
    reference's u array: (nodes, 3), node n = i + (N+1) j + (N+1)^2 k."""
    h = np.asarray(lengths, dtype=float) / N
    N1 = N + 1
    nodes = N1 ** 3
    vol = h.prod()
    gp = 1 / np.sqrt(3.0)
    Ke = np.zeros((8, 8))
    for p in [(x, y, z) for x in (-gp, gp) for y in (-gp, gp) for z in (-gp, gp)]:
        B = element_grad(p, h)
        Ke += (vol / 8) * B @ B.T          # weight 1 x Jdet (h/2)^3
    Bc = element_grad((0.0, 0.0, 0.0), h) * vol  # one point, weight 8 x Jdet
    rows, cols, vals = [], [], []
    b = np.zeros((nodes, 3))
    F9 = F.reshape(9, N, N, N)               # [comp, c(x), b(y), a(z)]
    for i in range(N):
        for j in range(N):
            for k in range(N):
                n0 = i + N1 * j + N1 * N1 * k
                conn = [n0 + (s[0] > 0) + N1 * (s[1] > 0) + N1 * N1 * (s[2] > 0) for s in _SIGNS]
                Fe = F9[:, i, j, k].reshape(3, 3)   # F_rj
                be = Bc @ Fe.T                       # (8, 3): sum_j dN/dX_j F_rj
                for a in range(8):
                    b[conn[a]] += be[a]
                    for c in range(8):
                        rows.append(conn[a]); cols.append(conn[c]); vals.append(Ke[a, c])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(nodes, nodes))
    A1 = A[1:, 1:].tocsc()
    x = np.zeros((nodes, 3))
    for r in range(3):
        x[1:, r] = spla.spsolve(A1, b[1:, r])
    idx = np.arange(nodes)
    X = np.stack([(idx % N1) * h[0], (idx // N1 % N1) * h[1], (idx // (N1 * N1)) * h[2]], axis=1)
    u = x - X
    u[0] = 0.0
    return u
