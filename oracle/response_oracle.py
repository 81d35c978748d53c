"""TEST INFRASTRUCTURE ONLY -- never imported by the product.

CPU restatement of the reference's impact-zone collision response, used to
check the product's (csrc/ys_zones.h, driven by the GPU detection in
csrc/ys_collide.cu):

- collision_response's round loop, the velocity update and the active
  faces of update_active (src/Collision.cpp:73-182);
- the time order of impacts (operator<, src/Collision.cpp:255-257) and the
  greedy independent subset (indenpendent_impacts / conflict,
  src/Collision.cpp:259-283);
- add_impacts / find_or_create_zone / merge_zone with the reference's
  vector order (src/Collision.cpp:438-476);
- the zone projection of NormalOpt (src/Collision.cpp:684-740,
  src/Collision.h:139-165): min 1/2 sum a_i |x_i - x_old_i|^2 subject to
  sum_k w_k n . x_k >= thickness, a_i = inv_m m_i;
- the derivative of one projection (precompute_derivative and
  compute_derivative, src/Collision.cpp:478-524, 602-674).

Parity is unpinned against the reference's own numbers: it solves each
projection with an augmented Lagrangian over Alglib's nonlinear CG
(src/AugLag.cpp:13-43) and Alglib is not part of the reference tree, so
neither its iterates nor its tolerances can be reproduced here. The
restatement solves the projection exactly (a least-distance programme through
scipy's non-negative least squares) and the tests pin it by its optimality
conditions. Ties in time, which the reference leaves to its thread order
and std::sort, are broken by (type, nodes, weights, normal).

Detection is a callback detect(x, face_active) -> list of impacts, each
(type, nodes[4], t, w[4], n[3]) with obstacle nodes as -1 - id.
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import nnls


def sort_key(im):
    typ, nodes, t, w, n = im
    return (t, typ, *[int(v) for v in nodes], *[float(v) for v in w], *[float(v) for v in n])


def independent(impacts):
    """Sorted by time, then greedy: an impact is dropped when one of its free
    nodes is a node of an impact already kept (conflict())."""
    kept = []
    for im in sorted(impacts, key=sort_key):
        if any(nd >= 0 and any(nd in k[1] for k in kept) for nd in im[1]):
            continue
        kept.append(im)
    return kept


def ldp(G, h):
    """min |u| s.t. G u >= h (Lawson and Hanson ch. 23, scipy's NNLS):
    (u, lam, feasible)."""
    k, n = G.shape
    s = max(float(np.max(h)), 0.0) if k else 0.0
    if s <= 0.0:
        return np.zeros(n), np.zeros(k), True
    E = np.vstack([G.T, (h / s)[None, :]])
    f = np.zeros(n + 1)
    f[n] = 1.0
    lam_hat, _ = nnls(E, f, maxiter=50 * max(k, 1))
    r = E @ lam_hat - f
    if not r[n] < -1e-12:
        return np.zeros(n), np.zeros(k), False
    u = s * (-r[:n] / r[n])
    return u, s * lam_hat / (-r[n]), True


def project(nodes, imps, accepted, x, xold, obs_x, thickness, mass):
    """One zone projection; returns the record the backward needs."""
    m = len(nodes)
    ms = np.array([1.0 if mass is None else mass[i] for i in nodes])
    inv_m = np.mean(1.0 / ms)
    a = inv_m * ms
    loc = {nd: i for i, nd in enumerate(nodes)}
    G = np.zeros((len(imps), 3 * m))
    h = np.zeros(len(imps))
    for j, idx in enumerate(imps):
        typ, nd4, t, w, n = accepted[idx]
        hj = thickness
        for q in range(4):
            nd = nd4[q]
            if nd >= 0:
                li = loc[nd]
                G[j, 3 * li:3 * li + 3] += w[q] * np.asarray(n) / np.sqrt(a[li])
                hj -= w[q] * np.dot(n, xold[nd])
            else:
                hj -= w[q] * np.dot(n, obs_x[-1 - nd])
        h[j] = hj
    u, lam, ok = ldp(G, h)
    out = np.array([xold[nd] + u[3 * i:3 * i + 3] / np.sqrt(a[i]) for i, nd in enumerate(nodes)]) if ok else \
        np.array([x[nd] for nd in nodes])
    for i, nd in enumerate(nodes):
        x[nd] = out[i]
    return dict(nodes=list(nodes), imps=list(imps), a=a, xout=out.reshape(-1), lam=lam, feasible=ok, G=G, h=h, u=u)


def respond(x, faces, detect, thickness, h, damp, obs_x=None, v=None, mass=None, max_iter=100):
    """collision_response(damp) over positions x [n, 3]; returns dict(x, v,
    rounds, converged, changed, zones, accepted, rounds_of, tape)."""
    x = np.array(x, dtype=np.float64).reshape(-1, 3).copy()
    xold = x.copy()
    obs_x = np.zeros((0, 3)) if obs_x is None else np.asarray(obs_x, np.float64).reshape(-1, 3)
    faces = np.asarray(faces).reshape(-1, 3)
    node_faces = [[] for _ in range(len(x))]
    for f, tri in enumerate(faces):
        for nd in tri:
            node_faces[int(nd)].append(f)
    zones = []  # [nodes, imps, active], the reference's vector order
    accepted, rounds_of, tape = [], [], []
    changed = False

    def find_or_create(nd):
        for z in zones:
            if nd in z[0]:
                return z
        z = [[nd], [], False]
        zones.append(z)
        return z

    it = 0
    while it < max_iter:
        mask = None
        if zones:
            mask = np.zeros(len(faces), np.uint8)
            for z in zones:
                if z[2]:
                    for nd in z[0]:
                        mask[node_faces[nd]] = 1
        found = detect(x, mask)
        indep = independent(found)
        if not indep:
            break
        for z in zones:
            z[2] = False
        for im in indep:
            idx = len(accepted)
            accepted.append(im)
            rounds_of.append(it)
            nd4 = im[1]
            zone = find_or_create(nd4[0] if nd4[0] >= 0 else nd4[3])
            for nd in nd4:
                if nd >= 0:
                    other = find_or_create(nd)
                    if other is not zone:
                        zone[0] += other[0]
                        zone[1] += other[1]
                        zones.remove(other)
            zone[1].append(idx)
            zone[2] = True
        for z in zones:
            if z[2]:
                changed = True
                tape.append(project(z[0], z[1], accepted, x, xold, obs_x, thickness, mass))
        it += 1
    vout = None
    if v is not None:
        vout = np.array(v, np.float64).reshape(-1, 3).copy()
        if changed:
            vout = vout + (damp * (x - xold)) / h
    return dict(x=x, v=vout, rounds=it, converged=it < max_iter, changed=changed, zones=len(zones),
                accepted=accepted, rounds_of=rounds_of, tape=tape)


def projection_backward(rec, accepted, obs_x, thickness, gz):
    """The reference's derivative of one projection: gz = dL/dx_out of the
    zone's nodes [3m]; returns (dL/dx_in [3m], {impact: (dL/dw[4], dL/dn[3])})."""
    nodes, imps = rec["nodes"], rec["imps"]
    m = len(nodes)
    loc = {nd: i for i, nd in enumerate(nodes)}
    xout = rec["xout"]
    sm1 = np.repeat(1.0 / np.sqrt(rec["a"]), 3)
    legal = []
    for j, idx in enumerate(imps):
        typ, nd4, t, w, n = accepted[idx]
        c = thickness
        for q in range(4):
            xq = xout[3 * loc[nd4[q]]:3 * loc[nd4[q]] + 3] if nd4[q] >= 0 else obs_x[-1 - nd4[q]]
            c -= w[q] * np.dot(n, xq)
        if c >= -1e-6:
            legal.append(j)
    L = len(legal)
    A = np.zeros((3 * m, L))
    for l, j in enumerate(legal):
        typ, nd4, t, w, n = accepted[imps[j]]
        for q in range(4):
            if nd4[q] >= 0:
                li = loc[nd4[q]]
                A[3 * li:3 * li + 3, l] -= w[q] * np.asarray(n) * sm1[3 * li:3 * li + 3]
    lam = np.array(rec["lam"], np.float64).copy()
    if L:
        Q, R = np.linalg.qr(A, mode="reduced" if L <= 3 * m else "complete")
        cols = min(L, 3 * m)
        nd0 = 0
        while nd0 < cols and abs(R[nd0, nd0]) >= 1e-6:
            nd0 += 1
        Q0, R0 = Q[:, :nd0], R[:nd0, :nd0]
        if nd0:
            r1l = R[:nd0, nd0:L] @ lam[[legal[l] for l in range(nd0, L)]] if L > nd0 else np.zeros(nd0)
            lamp = np.linalg.solve(R0, r1l)
            for i in range(nd0):
                lam[legal[i]] += lamp[i]
        for l in range(nd0, L):
            lam[legal[l]] = 0.0
    else:
        nd0 = 0
        Q0, R0 = np.zeros((3 * m, 0)), np.zeros((0, 0))
    qtx = Q0.T @ (gz * sm1)
    dz = sm1 * (sm1 * gz - Q0 @ qtx)
    dlam = np.zeros(len(imps))
    if nd0:
        d0 = np.linalg.solve(R0, qtx)
        for i in range(nd0):
            dlam[legal[i]] = d0[i]
    grads = {}
    for j, idx in enumerate(imps):
        typ, nd4, t, w, n = accepted[idx]
        gw, gn = np.zeros(4), np.zeros(3)
        for q in range(4):
            if nd4[q] >= 0:
                li = loc[nd4[q]]
                tv = dlam[j] * xout[3 * li:3 * li + 3] + lam[j] * dz[3 * li:3 * li + 3]
            else:
                tv = dlam[j] * obs_x[-1 - nd4[q]]
            gw[q] += np.dot(tv, n)
            gn += w[q] * tv
        grads[idx] = (gw, gn)
    return dz / sm1 ** 2, grads


def respond_backward(res, obs_x, thickness, h, damp, gx, gv=None):
    """Backward of respond(): gx, gv = dL/dx, dL/dv after the response;
    returns (dL/dx before, dL/dv before, dL/dw [A, 4], dL/dn [A, 3])."""
    obs_x = np.zeros((0, 3)) if obs_x is None else np.asarray(obs_x, np.float64).reshape(-1, 3)
    g = np.array(gx, np.float64).reshape(-1, 3).copy()
    k = damp / h
    if gv is not None and res["changed"]:
        g += k * np.asarray(gv).reshape(-1, 3)
    A = len(res["accepted"])
    gw, gn = np.zeros((A, 4)), np.zeros((A, 3))
    for rec in reversed(res["tape"]):
        nodes = rec["nodes"]
        gz = g[nodes].reshape(-1)
        gin, grads = projection_backward(rec, res["accepted"], obs_x, thickness, gz)
        g[nodes] = gin.reshape(-1, 3)
        for idx, (a, b) in grads.items():
            gw[idx] += a
            gn[idx] += b
    if gv is not None and res["changed"]:
        g -= k * np.asarray(gv).reshape(-1, 3)
    gvin = np.zeros_like(g) if gv is None else np.asarray(gv, np.float64).reshape(-1, 3).copy()
    return g, gvin, gw, gn


def kkt_residual(rec, thickness, obs_x, accepted, xold):
    """Max violation of the projection's optimality conditions (primal
    feasibility, dual feasibility, complementarity, stationarity), scaled by
    the thickness."""
    G, h, u, lam = rec["G"], rec["h"], rec["u"], rec["lam"]
    if not len(h):
        return 0.0
    slack = G @ u - h
    r = [max(0.0, -slack.min()), max(0.0, -lam.min()), np.abs(lam * slack).max() / max(1.0, lam.max()),
         np.abs(u - G.T @ lam).max()]
    return max(r) / thickness
