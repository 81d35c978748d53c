"""Test helper: the structured stencil storage of one cloth's row blocks
(csrc/ys_common.cuh) expanded into the reference's dense DOF layout."""
import numpy as np

DU = [0, -1, 1, 0, 0, -2, 2, 0, 0, -1, 1, -1, 1]
DV = [0, 0, 0, -1, 1, 0, 0, -2, 2, -1, -1, 1, 1]
LL, LE_SELF, EL_SELF, EE_SELF, LE_NBR, EL_NBR, EE_NBR, NSLOTS = 0, 117, 123, 129, 131, 143, 155, 159
NBR = [(-1, 0, 0), (1, 0, 0), (0, -1, 1), (0, 1, 1)]  # (du, dv, k)


def slots_to_dense(slots, rhs, W, H):
    """slots [159][N], rhs [5][N] (node order u + v*W) -> (A, b) reference layout."""
    N = W * H
    dim = 3 * N + 2 * (W - 2) * (H - 2)
    A = np.zeros((dim, dim))
    b = np.zeros(dim)

    def interior(u, v):
        return 0 < u < W - 1 and 0 < v < H - 1

    def erow(u, v):
        return 3 * N + 2 * ((u - 1) + (v - 1) * (W - 2))

    for v in range(H):
        for u in range(W):
            n = u + v * W
            b[3 * n:3 * n + 3] = rhs[0:3, n]
            for s in range(13):
                uu, vv = u + DU[s], v + DV[s]
                if not (0 <= uu < W and 0 <= vv < H):
                    continue
                j = uu + vv * W
                A[3 * n:3 * n + 3, 3 * j:3 * j + 3] = slots[LL + 9 * s:LL + 9 * s + 9, n].reshape(3, 3)
            if not interior(u, v):
                continue
            er = erow(u, v)
            b[er:er + 2] = rhs[3:5, n]
            A[3 * n:3 * n + 3, er:er + 2] = slots[LE_SELF:LE_SELF + 6, n].reshape(3, 2)
            A[er:er + 2, 3 * n:3 * n + 3] = slots[EL_SELF:EL_SELF + 6, n].reshape(2, 3)
            A[er, er] = slots[EE_SELF, n]
            A[er + 1, er + 1] = slots[EE_SELF + 1, n]
            for m, (du, dv, k) in enumerate(NBR):
                uu, vv = u + du, v + dv
                if not interior(uu, vv):
                    continue
                j = uu + vv * W
                ej = erow(uu, vv)
                A[3 * n:3 * n + 3, ej + k] = slots[LE_NBR + 3 * m:LE_NBR + 3 * m + 3, n]
                A[er + k, 3 * j:3 * j + 3] = slots[EL_NBR + 3 * m:EL_NBR + 3 * m + 3, n]
                A[er + k, ej + k] = slots[EE_NBR + m, n]
    return A, b


def node5_to_ref(x5, W, H):
    """[N][5] node-layout vector -> reference DOF vector."""
    N = W * H
    out = np.zeros(3 * N + 2 * (W - 2) * (H - 2))
    out[:3 * N] = x5[:, :3].reshape(-1)
    for v in range(1, H - 1):
        for u in range(1, W - 1):
            n = u + v * W
            e = 3 * N + 2 * ((u - 1) + (v - 1) * (W - 2))
            out[e:e + 2] = x5[n, 3:5]
    return out


def ref_to_node5(xr, W, H):
    N = W * H
    out = np.zeros((N, 5))
    out[:, :3] = xr[:3 * N].reshape(N, 3)
    for v in range(1, H - 1):
        for u in range(1, W - 1):
            n = u + v * W
            e = 3 * N + 2 * ((u - 1) + (v - 1) * (W - 2))
            out[n, 3:5] = xr[e:e + 2]
    return out
