"""Canonical comparisons between the CUDA library and the oracle.

Tolerances (stated once, used by the parity tests and the benchmark's error
report):
  FIELD_TOL_FP64  field values against the FP64 oracle (same float inputs,
              double arithmetic): |f_gpu - f_64| <= FIELD_TOL_FP64 * MaxScalar.
  FIELD_TOL   field values against the float oracle: the reference's own
              float arithmetic is up to ~1.1e-5 * MaxScalar off the FP64
              answer (G from a float SVD, naive float sums), so the bound is
              the sum of both errors.
  XMEAN_TOL   smoothed centres: |dx| <= XMEAN_TOL * r.
  G_TOL       anisotropy matrices (entries O(1)) and determinants.
  NORMAL_TOL  particle normals relative to the largest normal of the frame.
  VERT_TOL    mesh vertex positions: |dp| <= VERT_TOL * r.
  ISO_EPS     a sample whose oracle value is within ISO_EPS * MaxScalar of
              zero may take the other sign (counted, reported).
  CURV_EPS    a node whose curvature is within CURV_EPS of 0.99 may be
              classified the other way (counted, reported).
"""
import numpy as np

FIELD_TOL_FP64 = 1e-5
FIELD_TOL = 3e-5
XMEAN_TOL = 1e-4
G_TOL = 1e-4
NORMAL_TOL = 1e-4
VERT_TOL = 1e-3
ISO_EPS = 1e-5
CURV_EPS = 1e-4


def sample_points(center, half):
    """TNode::GenerateSampling (src/iso_method_ours.cpp:52-75) in float32."""
    c = np.asarray(center, np.float32)
    h = np.float32(half)
    mn = c - h
    mx = c + h
    pts = np.empty((27, 3), np.float32)
    for z in range(3):
        for y in range(3):
            for x in range(3):
                i = z * 9 + y * 3 + x
                t = np.array([x, y, z], np.float32) / np.float32(2)
                pts[i] = (np.float32(1) - t) * mn + t * mx
    return pts


def node_table(nodes, fields=("type", "node", "curv", "signchange")):
    """dict (depth, id) -> record, from an oracle nodes() dict or a GPU pi_node array."""
    out = {}
    if isinstance(nodes, dict):
        for i in range(len(nodes["id"])):
            out[(int(nodes["depth"][i]), int(nodes["id"][i]))] = (
                int(nodes["type"][i]), nodes["node"][i], float(nodes["curv"][i]), int(nodes["signchange"][i]),
                nodes["center"][i], float(nodes["half"][i]))
    else:
        for r in nodes:
            out[(int(r["depth"]), int(r["id"]))] = (int(r["type"]), r["node"], float(r["curv"]),
                                                   int(r["signchange"]), r["center"], float(r["half"]))
    return out


def compare_octrees(o_nodes, g_nodes, oracle, max_scalar, depth_min):
    """Node-by-node comparison keyed by (depth, id).  Returns a report dict:
    mismatched classifications, of which how many are explained by a sample
    within ISO_EPS of the isovalue or a curvature within CURV_EPS of 0.99
    (their subtrees are then skipped), and the max leaf-value difference."""
    A = node_table(o_nodes)
    B = node_table(g_nodes)
    rep = dict(nodes_oracle=len(A), nodes_gpu=len(B), type_mismatch=0, explained=0, unexplained=[],
               leaf_value_maxdiff=0.0, compared=0)
    far_pos, far_gpu = [], []
    skip_prefix = set()

    def under_skipped(key):
        d, i = key
        while d > 0:
            d -= 1
            i //= 8
            if (d, i) in skip_prefix:
                return True
        return False

    for key in sorted(A, key=lambda k: k[0]):
        if under_skipped(key):
            continue
        if key not in B:
            rep["unexplained"].append(("missing", key))
            continue
        ta, na, ca, sa, cen, half = A[key]
        tb, nb, cb, sb, _, _ = B[key]
        rep["compared"] += 1
        if ta != tb:
            rep["type_mismatch"] += 1
            near = abs(ca - 0.99) < CURV_EPS
            if not near and key[0] >= depth_min:
                vals = oracle.eval(sample_points(cen, half))
                near = np.min(np.abs(vals)) < ISO_EPS * max_scalar
            if near:
                rep["explained"] += 1
                skip_prefix.add(key)
            else:
                rep["unexplained"].append(("type", key, ta, tb, ca, cb, sa, sb))
            continue
        if ta == 2:
            dv = abs(float(na[3]) - float(nb[3]))
            rep["leaf_value_maxdiff"] = max(rep["leaf_value_maxdiff"], dv)
            if dv > FIELD_TOL * max_scalar:
                far_pos.append(np.asarray(nb[:3], np.float32))
                far_gpu.append(float(nb[3]))
    for key in B:
        if key not in A and not under_skipped(key):
            rep["unexplained"].append(("extra", key))
    rep["leaf_far_pos"] = np.array(far_pos, np.float32).reshape(-1, 3)
    rep["leaf_far_gpu"] = np.array(far_gpu)
    return rep


def canonical_mesh(verts, tris, vkeys, one_based):
    """Vertices keyed by their sorted leaf-id pair; triangles as rotated
    triples of vertex keys (orientation kept, rotation normalised)."""
    t = np.asarray(tris, np.int64) - (1 if one_based else 0)
    keys = [(int(a), int(b)) for a, b in vkeys]
    vmap = {k: verts[i] for i, k in enumerate(keys)}
    tri = set()
    for a, b, c in t:
        ka, kb, kc = keys[a], keys[b], keys[c]
        rots = [(ka, kb, kc), (kb, kc, ka), (kc, ka, kb)]
        tri.add(min(rots))
    return vmap, tri


def compare_meshes(o_mesh, g_mesh, radius):
    ov, ot, ok = o_mesh
    gv, gt, gk = g_mesh
    vo, to = canonical_mesh(ov, ot, ok, True)
    vg, tg = canonical_mesh(gv, gt, gk, False)
    common = set(vo) & set(vg)
    d = np.array([np.max(np.abs(vo[k] - vg[k])) for k in common]) if common else np.zeros(1)
    rep = dict(verts_oracle=len(vo), verts_gpu=len(vg), verts_only_oracle=len(set(vo) - set(vg)),
               verts_only_gpu=len(set(vg) - set(vo)), tris_oracle=len(to), tris_gpu=len(tg),
               tris_only_oracle=len(to - tg), tris_only_gpu=len(tg - to),
               vert_maxdiff_over_r=float(d.max() / radius), vert_rmsdiff_over_r=float(np.sqrt(np.mean(d ** 2)) / radius),
               verts_off_tol=int(np.sum(d > VERT_TOL * radius)))
    return rep


QEF_VERT_TOL = 1e-4  # QEF vertex vs the FP64 solve of the same samples, in units of r


def qef_solve_f64(center, half, samples):
    """TNode::NodeCalcNode (src/iso_method_ours.cpp:101-174) in float64 with the
    library's rule (diagonal equilibration, eigen pseudo-inverse, relative
    threshold 1e-12): returns (x[4], in_cell, singular, err)."""
    c = np.asarray(center, np.float32)
    h = np.float32(half)
    mn = c - h
    mx = c + h
    pts = sample_points(center, half).astype(np.float64)
    f = np.asarray(samples, np.float64)
    step = np.float64(np.float32(2.0) * h / np.float32(2))
    v = f.reshape(3, 3, 3)  # [z, y, x]
    g = np.zeros((3, 3, 3, 3))
    for ax, axis in ((0, 2), (1, 1), (2, 0)):  # gradient component ax differentiates array axis `axis`
        vv = np.moveaxis(v, axis, 0)
        gg = np.empty_like(vv)
        gg[0] = (vv[0] - vv[1]) / step
        gg[2] = (vv[1] - vv[2]) / step
        gg[1] = (vv[0] - vv[2]) / (2 * step)
        g[..., ax] = np.moveaxis(gg, 0, axis)
    g = g.reshape(27, 3)
    pl = np.concatenate([g, -np.ones((27, 1)), (-(pts * g).sum(1) + f)[:, None]], axis=1)
    M = pl.T @ pl
    A = M[:4, :4]
    B = -M[:4, 4]
    d = np.where(np.diag(A) > 0, 1.0 / np.sqrt(np.where(np.diag(A) > 0, np.diag(A), 1.0)), 1.0)
    As = A * d[:, None] * d[None, :]
    w, V = np.linalg.eigh(As)
    tol = 1e-12 * np.abs(w).max() if np.abs(w).max() > 0 else 0.0
    keep = np.abs(w) > tol
    singular = not keep.all()
    x = d * (V[:, keep] @ ((V[:, keep].T @ (d * B)) / w[keep]))
    in_cell = bool(np.all(x[:3] >= mn) and np.all(x[:3] <= mx))
    err = float(np.sum((g @ x[:3] - (pts * g).sum(1) - x[3]) ** 2 / (1 + (g * g).sum(1))))
    return x, in_cell, singular, err


# ---------------------------------------------------------------------------
# Vectorised forms of the comparisons above, for frames of millions of nodes
# (the headline configurations).  Same rules and bounds.
# ---------------------------------------------------------------------------

def node_keys(depth, ids):
    """(depth, id) -> one uint64 (depth in the top 5 bits; ids < 8^19)."""
    d = np.asarray(depth).astype(np.uint64)
    i = np.asarray(ids).astype(np.uint64)
    assert d.size == 0 or int(d.max()) < 20
    return (d << np.uint64(59)) | i


def _under(keys_depth, keys_id, skip):
    """Mask of nodes (depth, id arrays) strictly below one of the skip nodes."""
    mask = np.zeros(len(keys_depth), bool)
    if not skip:
        return mask
    sk = np.array(skip, dtype=np.int64)
    d = keys_depth.astype(np.int64)
    ids = keys_id.astype(np.uint64)
    for d0 in np.unique(sk[:, 0]):
        sel = d > d0
        if not sel.any():
            continue
        anc = ids[sel] >> (np.uint64(3) * (d[sel] - d0).astype(np.uint64))
        want = np.array(sorted(set(int(x) for x in sk[sk[:, 0] == d0, 1])), np.uint64)
        mask[np.nonzero(sel)[0][np.isin(anc, want)]] = True
    return mask


def compare_octrees_fast(o_nodes, g_nodes, oracle, max_scalar, depth_min, fp64_eval=None):
    """compare_octrees over arrays.  o_nodes: the oracle's nodes() dict;
    g_nodes: the library's pi_node dump.  A type mismatch is explained when a
    curvature lies within CURV_EPS of 0.99 or (at depth >= D_min) a sample of
    the node lies within ISO_EPS * MaxScalar of the isovalue (oracle values);
    its subtree is then skipped.  Leaf values beyond FIELD_TOL * MaxScalar of
    the float oracle must be within FIELD_TOL_FP64 of fp64_eval (when given)."""
    od, oi, ot = o_nodes["depth"], o_nodes["id"], o_nodes["type"]
    gd, gi, gt = g_nodes["depth"], g_nodes["id"], g_nodes["type"]
    ka = node_keys(od, oi)
    kb = node_keys(gd, gi)
    assert len(np.unique(ka)) == len(ka) and len(np.unique(kb)) == len(kb)
    common, ia, ib = np.intersect1d(ka, kb, assume_unique=True, return_indices=True)
    rep = dict(nodes_oracle=len(ka), nodes_gpu=len(kb), type_mismatch=0, explained=0, unexplained=[],
               leaf_value_maxdiff=0.0, compared=0, leaves_beyond_float_tol=0, leaf_far_vs_fp64_max=0.0)
    mism = np.nonzero(ot[ia] != gt[ib])[0]
    mism = mism[np.argsort(od[ia[mism]], kind="stable")]
    rep["type_mismatch"] = int(len(mism))
    skip = []
    for m in mism:
        a, b = ia[m], ib[m]
        d, i = int(od[a]), int(oi[a])
        if any(d > d0 and (i >> (3 * (d - d0))) == i0 for d0, i0 in skip):
            continue
        ca, cb = float(o_nodes["curv"][a]), float(g_nodes["curv"][b])
        near = abs(ca - 0.99) < CURV_EPS
        if not near and d >= depth_min:
            vals = oracle.eval(sample_points(o_nodes["center"][a], o_nodes["half"][a]))
            near = np.min(np.abs(vals)) < ISO_EPS * max_scalar
        if near:
            rep["explained"] += 1
            skip.append((d, i))
        else:
            rep["unexplained"].append(("type", (d, i), int(ot[a]), int(gt[b]), ca, cb))
    only_a = np.setdiff1d(np.arange(len(ka)), ia, assume_unique=True)
    only_b = np.setdiff1d(np.arange(len(kb)), ib, assume_unique=True)
    for idx, dd, ii, tag in ((only_a, od, oi, "missing"), (only_b, gd, gi, "extra")):
        bad = idx[~_under(dd[idx], ii[idx], skip)]
        rep["unexplained"] += [(tag, (int(dd[k]), int(ii[k]))) for k in bad[:20]]
        if len(bad) > 20:
            rep["unexplained"].append((tag, "%d more" % (len(bad) - 20)))
    live = ~_under(od[ia], oi[ia], skip)
    rep["compared"] = int(live.sum())
    leaf = live & (ot[ia] == 2) & (gt[ib] == 2)
    va = o_nodes["node"][ia[leaf], 3].astype(np.float64)
    vb = g_nodes["node"][ib[leaf]][:, 3].astype(np.float64)
    dv = np.abs(va - vb)
    rep["leaf_value_maxdiff"] = float(dv.max()) if len(dv) else 0.0
    far = dv > FIELD_TOL * max_scalar
    rep["leaves_beyond_float_tol"] = int(far.sum())
    if far.any() and fp64_eval is not None:
        pos = g_nodes["node"][ib[leaf][far]][:, :3].astype(np.float32)
        v64 = fp64_eval(pos)
        rep["leaf_far_vs_fp64_max"] = float((np.abs(vb[far] - v64) / max_scalar).max())
    return rep


def _pair_view(k):
    k = np.ascontiguousarray(np.asarray(k, np.uint64).reshape(-1, 2))
    return k.view([("a", "<u8"), ("b", "<u8")]).ravel()


def _tri_view(t):
    """Triangles (n, 3) of global vertex ids, rotated so that the smallest id
    comes first (orientation kept), as a structured array for set operations."""
    t = np.asarray(t, np.int64).reshape(-1, 3)
    r = np.argmin(t, axis=1)
    rows = np.arange(len(t))
    out = np.stack([t[rows, r], t[rows, (r + 1) % 3], t[rows, (r + 2) % 3]], 1)
    out = np.ascontiguousarray(out)
    return out.view([("a", "<i8"), ("b", "<i8"), ("c", "<i8")]).ravel()


def compare_meshes_fast(o_mesh, g_mesh, radius):
    """compare_meshes over arrays: vertices keyed by their leaf-id pair,
    triangles as rotated triples of vertex keys."""
    ov, ot, ok = o_mesh
    gv, gt, gk = g_mesh
    allk = np.concatenate([_pair_view(ok), _pair_view(gk)])
    uniq, inv = np.unique(allk, return_inverse=True)
    io, ig = inv[:len(ok)], inv[len(ok):]
    assert len(np.unique(io)) == len(io) and len(np.unique(ig)) == len(ig)
    so = np.zeros(len(uniq), bool)
    sg = np.zeros(len(uniq), bool)
    so[io] = True
    sg[ig] = True
    po = np.zeros((len(uniq), 3), np.float32)
    pg = np.zeros((len(uniq), 3), np.float32)
    po[io] = ov
    pg[ig] = gv
    both = so & sg
    d = np.abs(po[both] - pg[both]).max(1) if both.any() else np.zeros(1)
    to = np.unique(_tri_view(io[np.asarray(ot, np.int64) - 1]))
    tg = np.unique(_tri_view(ig[np.asarray(gt, np.int64)]))
    tc = np.intersect1d(to, tg, assume_unique=True)
    # GPU vertices present in both meshes but off the float oracle's by more
    # than the tolerance (indices into the GPU mesh), for arbitrate_vertices
    gd = np.zeros(len(gv))
    gb = so[ig]
    gd[gb] = np.abs(po[ig[gb]] - gv[gb]).max(1)
    return dict(verts_oracle=int(so.sum()), verts_gpu=int(sg.sum()), verts_only_oracle=int((so & ~sg).sum()),
                verts_only_gpu=int((sg & ~so).sum()), tris_oracle=len(to), tris_gpu=len(tg),
                tris_only_oracle=len(to) - len(tc), tris_only_gpu=len(tg) - len(tc),
                vert_maxdiff_over_r=float(d.max() / radius),
                vert_rmsdiff_over_r=float(np.sqrt(np.mean(d.astype(np.float64) ** 2)) / radius),
                verts_off_tol=int(np.sum(d > VERT_TOL * radius)),
                off_gpu_idx=np.flatnonzero(gd > VERT_TOL * radius))


def _fnorm(dx, dy, dz):
    """|d| rounded as the library's bisection rounds it (float32,
    x^2 + (y^2 + z^2), then sqrt)."""
    return np.sqrt(dx * dx + (dy * dy + dz * dz)).astype(np.float32)


def bisect_fp64(p, q, rr, eval64, max_scalar):
    """The edge bisection of calc_vertices (src/visitorextract.cpp:41-93), as
    the library runs it (float midpoints, halved float length, stop at
    length <= rr, lerp with the 0.1 / 0.9 snap), with every midpoint value
    from the FP64 oracle, for many edges at once.  p, q: float32 (n, 4) node
    points (xyz, value) of the two leaves.  Returns the FP64 vertex (n, 3),
    and for each edge whether a decision was a near tie: a midpoint value
    within 2 FIELD_TOL_FP64 * MaxScalar of zero, or a lerp ratio whose
    distance to a snap threshold is within what that error moves it; and the
    distance that error moves the lerped vertex."""
    p = np.asarray(p, np.float32).copy()
    q = np.asarray(q, np.float32).copy()
    pw = p[:, 3].astype(np.float64)
    qw = q[:, 3].astype(np.float64)
    n = len(p)
    d = _fnorm(p[:, 0] - q[:, 0], p[:, 1] - q[:, 1], p[:, 2] - q[:, 2])
    rr = np.float32(rr)
    tie = np.zeros(n, bool)
    band = 2 * FIELD_TOL_FP64 * max_scalar
    for _ in range(64):
        act = d > rr
        if not act.any():
            break
        m = ((p[act, :3] + q[act, :3]) * np.float32(0.5)).astype(np.float32)
        mw = eval64(m)
        tie[np.flatnonzero(act)[np.abs(mw) < band]] = True
        keep_p = (mw > 0) == (pw[act] > 0)
        ia = np.flatnonzero(act)
        tp, tq = ia[keep_p], ia[~keep_p]
        p[tp, :3], pw[tp] = m[keep_p], mw[keep_p]
        q[tq, :3], qw[tq] = m[~keep_p], mw[~keep_p]
        d[act] = (d[act] * np.float32(0.5)).astype(np.float32)
    den = qw - pw
    ratio = -pw / den
    dr = band / np.maximum(np.abs(den), 1e-300)
    tie |= (np.abs(ratio - 0.1) < dr) | (np.abs(ratio - 0.9) < dr)
    P, Q = p[:, :3].astype(np.float64), q[:, :3].astype(np.float64)
    v = P + (Q - P) * ratio[:, None]
    v[ratio < 0.1] = P[ratio < 0.1]
    v[ratio > 0.9] = Q[ratio > 0.9]
    slack = np.linalg.norm(Q - P, axis=1) * dr
    return v, tie, slack


def check_vertices_fp64(g, m, radius, max_scalar, dump_nodes, dump_edges):
    """arbitrate_vertices for a library frame g (a constant radius: the
    bisection stops at r / 2) and the report m of compare_meshes_fast; the
    dump codes are the library's PI_DUMP_NODES and PI_DUMP_VERTEX_EDGES."""
    gv = g.mesh()[0]
    rr = np.float32(radius) / np.float32(2)
    return arbitrate_vertices(g.dump(dump_nodes), g.dump(dump_edges), gv, m["off_gpu_idx"], rr, g.eval_fp64,
                              max_scalar, radius)


def arbitrate_vertices(g_nodes, edges, gv, idx, rr, eval64, max_scalar, radius):
    """GPU vertices idx that differ from the float oracle's by more than
    VERT_TOL * r, against the FP64 bisection of the same edge (bisect_fp64):
    each must lie within VERT_TOL * r (plus what the FP64 tolerance moves the
    lerp) of the FP64 vertex, or have a near-tie decision on its FP64 chain.
    Returns (agree, explained, unexplained indices)."""
    idx = np.asarray(idx, np.int64)
    if len(idx) == 0:
        return 0, 0, idx
    nv = g_nodes["node"]
    e = edges[idx]
    p, q = nv[e[:, 0]], nv[e[:, 1]]
    v64, tie, slack = bisect_fp64(p, q, rr, eval64, max_scalar)
    dist = np.abs(gv[idx].astype(np.float64) - v64).max(1)
    ok = dist <= VERT_TOL * radius + slack
    return int(ok.sum()), int((~ok & tie).sum()), idx[~ok & ~tie]


def qef_solve_f64_batch(centers, halves, samples):
    """qef_solve_f64 for many leaves at once: returns x [n, 4], in_cell [n],
    singular [n]."""
    c = np.asarray(centers, np.float32).reshape(-1, 3)
    h = np.asarray(halves, np.float32).reshape(-1)
    n = len(c)
    mn = c - h[:, None]
    mx = c + h[:, None]
    t = np.array([[x, y, z] for z in range(3) for y in range(3) for x in range(3)], np.float32) / np.float32(2)
    pts = ((np.float32(1) - t)[None] * mn[:, None, :] + t[None] * mx[:, None, :]).astype(np.float64)
    f = np.asarray(samples, np.float64).reshape(n, 27)
    step = (np.float32(2.0) * h / np.float32(2)).astype(np.float64)[:, None, None]
    v = f.reshape(n, 3, 3, 3)  # [node, z, y, x]
    g = np.zeros((n, 3, 3, 3, 3))
    for ax, axis in ((0, 3), (1, 2), (2, 1)):
        vv = np.moveaxis(v, axis, 1)
        gg = np.empty_like(vv)
        gg[:, 0] = (vv[:, 0] - vv[:, 1]) / step
        gg[:, 2] = (vv[:, 1] - vv[:, 2]) / step
        gg[:, 1] = (vv[:, 0] - vv[:, 2]) / (2 * step)
        g[..., ax] = np.moveaxis(gg, 1, axis)
    g = g.reshape(n, 27, 3)
    pl = np.concatenate([g, -np.ones((n, 27, 1)), (-(pts * g).sum(2) + f)[:, :, None]], axis=2)
    M = np.einsum("nki,nkj->nij", pl, pl)
    A = M[:, :4, :4]
    B = -M[:, :4, 4]
    dg = np.diagonal(A, axis1=1, axis2=2)
    d = np.where(dg > 0, 1.0 / np.sqrt(np.where(dg > 0, dg, 1.0)), 1.0)
    As = A * d[:, :, None] * d[:, None, :]
    w, V = np.linalg.eigh(As)
    wmax = np.abs(w).max(1)
    keep = np.abs(w) > (1e-12 * wmax)[:, None]
    y = np.einsum("nji,nj->ni", V, d * B)
    y = np.where(keep, y / np.where(keep, w, 1.0), 0.0)
    x = d * np.einsum("nij,nj->ni", V, y)
    in_cell = np.all(x[:, :3] >= mn, axis=1) & np.all(x[:, :3] <= mx, axis=1)
    return x, in_cell, ~keep.all(1)
