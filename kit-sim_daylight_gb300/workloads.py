"""Seeded synthetic scenes for the engine's measured configurations and tests (host side, numpy).

Each scene is returned as the engine takes it at its boundary, after the reference's host prep: recentred float32
vertices and uint32 triangles (quads split 0-1-2 / 0-2-3, src/mesh.cpp:137-168), a global slot per triangle, and the
sensors (face centre + unit normal per sensor face, recentred: src/mesh.cpp:45-71, 315-349) in mesh order.

 - box_scene(): four 2 m ground quads at z 0 facing up on a 2 x 2 grid and a 1 m cube 0.5 m above the fourth, both
   sensor meshes that block (the reference's tests/box.obj, as its measured config describes it).
 - urban_block(): 20 x 20 extruded boxes, footprints U(10, 30) m, heights U(6, 60) m, street gaps U(5, 15) m (mt19937-
   style seeded numpy Generator, seed 42), roofs + facades remeshed into quads as receivers, a ground as context. The
   quad size is chosen, as the reference's own bench generator does (src/main.cpp:105: q = sqrt(area / nSens)), so that
   the block has ~200k sensor faces and ~400k triangles (1 m quads would give ~1.2M faces).
 - random_city(): small random box piles with optional porous / glass / thin-solid slots and labels, for parity tests.
"""
import numpy as np


class Mesh:
    """Accumulates quads (counter-clockwise seen from the side they face) into shared arrays."""

    def __init__(self, triangles=False):
        self.pts = []
        self.quads = []
        self.slot = []
        self.triangles = triangles   # faces are the quads' two triangles (0-1-2, 0-2-3): a sensor per triangle

    def grid(self, o, u, v, nu, nv, slot=0):
        o, u, v = (np.asarray(x, np.float64) for x in (o, u, v))
        b = sum(len(p) for p in self.pts)
        i = np.arange(nu + 1)[None, :, None] / nu
        j = np.arange(nv + 1)[:, None, None] / nv
        P = o + u * i + v * j
        self.pts.append(P.reshape(-1, 3))
        jj, ii = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
        a = (b + jj * (nu + 1) + ii).ravel()
        self.quads.append(np.stack([a, a + 1, a + nu + 2, a + nu + 1], axis=1))
        self.slot.append(np.full(nu * nv, slot, np.uint32))

    def arrays(self):
        pts = np.concatenate(self.pts) if self.pts else np.zeros((0, 3))
        q = np.concatenate(self.quads) if self.quads else np.zeros((0, 4), np.int64)
        s = np.concatenate(self.slot) if self.slot else np.zeros(0, np.uint32)
        return pts, q, s


def _faces_geom(pts, quads):
    """Centre (area-weighted over the two triangles) and unit normal of each quad, in double."""
    a, b, c, d = (pts[quads[:, k]] for k in range(4))
    n1 = np.cross(b - a, c - a)
    n2 = np.cross(c - a, d - a)
    A1 = 0.5 * np.linalg.norm(n1, axis=1)
    A2 = 0.5 * np.linalg.norm(n2, axis=1)
    c1 = (a + b + c) / 3
    c2 = (a + c + d) / 3
    cen = (c1 * A1[:, None] + c2 * A2[:, None]) / np.maximum(A1 + A2, 1e-300)[:, None]
    n = n1 + n2
    n /= np.maximum(np.linalg.norm(n, axis=1), 1e-300)[:, None]
    return cen, n


def assemble(meshes):
    """meshes: list of (Mesh, is_sensor, blocks). Returns the scene dict at the engine boundary."""
    arrs = [(m.arrays(), sensor, blocks) for m, sensor, blocks in meshes]
    m_of = {id(a[0][1]): m for a, (m, _, _) in zip(arrs, meshes)}
    allp = np.concatenate([a[0][0] for a in arrs if len(a[0][0])])
    centre = 0.5 * (allp.min(axis=0) + allp.max(axis=0))   # bbox centre of every mesh (src/mesh.cpp:107-118)
    V, T, S, P, N = [], [], [], [], []
    base = 0
    slot_base = 0
    for (pts, q, s), sensor, blocks in arrs:
        if blocks:
            V.append((pts - centre).astype(np.float32))
            T.append(np.concatenate([q[:, [0, 1, 2]], q[:, [0, 2, 3]]], axis=1).reshape(-1, 3) + base)
            S.append(np.repeat(s + slot_base, 2))
            base += len(pts)
        if sensor:
            if m_of[id(q)].triangles:   # each triangle a face: (a, b, c, c) is that triangle as a degenerate quad
                t = np.concatenate([q[:, [0, 1, 2, 2]], q[:, [0, 2, 3, 3]]], axis=1).reshape(-1, 4)
                c, n = _faces_geom(pts - centre, t)
            else:
                c, n = _faces_geom(pts - centre, q)
            P.append(c.astype(np.float32))
            N.append(n.astype(np.float32))
        slot_base += int(s.max()) + 1 if len(s) else 1
    return dict(v=np.concatenate(V), tri=np.concatenate(T).astype(np.uint32), slot=np.concatenate(S).astype(np.uint32),
                P=np.concatenate(P), N=np.concatenate(N), centre=centre)


def box_scene():
    ground, box = Mesh(), Mesh(triangles=True)
    for x0, y0 in [(-2, -2), (0, -2), (-2, 0), (0, 0)]:
        ground.grid((x0, y0, 0), (2, 0, 0), (0, 2, 0), 1, 1)
    lo, hi = 0.5, 1.5
    e = hi - lo
    for o, u, v in [((lo, lo, lo), (0, e, 0), (e, 0, 0)), ((lo, lo, hi), (e, 0, 0), (0, e, 0)),      # bottom (-z), top
                    ((lo, lo, lo), (e, 0, 0), (0, 0, e)), ((hi, lo, lo), (0, e, 0), (0, 0, e)),      # -y, +x
                    ((hi, hi, lo), (-e, 0, 0), (0, 0, e)), ((lo, hi, lo), (0, -e, 0), (0, 0, e))]:  # +y, -x
        box.grid(o, u, v, 1, 1)
    return assemble([(ground, True, True), (box, True, True)])


def _box_faces(m, x0, y0, w, d, h, q, slot=0, roof=True):
    """Facades (outward) and roof of an extruded box, remeshed into ~q-sized quads."""
    c = [(x0, y0), (x0 + w, y0), (x0 + w, y0 + d), (x0, y0 + d), (x0, y0)]   # counter-clockwise: outward walls
    for k in range(4):
        ux, uy = c[k + 1][0] - c[k][0], c[k + 1][1] - c[k][1]
        L = np.hypot(ux, uy)
        m.grid((c[k][0], c[k][1], 0), (ux, uy, 0), (0, 0, h), max(1, int(round(L / q))), max(1, int(round(h / q))), slot)
    if roof:
        m.grid((x0, y0, h), (w, 0, 0), (0, d, 0), max(1, int(round(w / q))), max(1, int(round(d / q))), slot)


def urban_block(seed=42, n=20, target_sensors=200_000, glass_share=0.0, glass_seed=7):
    """The 20 x 20 urban block. glass_share > 0 puts a share of the facade quads into slot 1 (glass windows)."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(10, 30, (n, n))
    d = rng.uniform(10, 30, (n, n))
    h = rng.uniform(6, 60, (n, n))
    gx = rng.uniform(5, 15, (n, n))
    gy = rng.uniform(5, 15, n)
    area = float(np.sum(2 * (w + d) * h + w * d))
    q = np.sqrt(area / target_sensors)
    rows_y = np.concatenate([[0.0], np.cumsum(d.max(axis=1) + gy)[:-1]])
    build = Mesh()
    for r in range(n):
        x = 0.0
        for k in range(n):
            _box_faces(build, x, rows_y[r], w[r, k], d[r, k], h[r, k], q)
            x += w[r, k] + gx[r, k]
    if glass_share > 0:
        g = np.random.default_rng(glass_seed)
        build.slot = [np.where(g.random(len(s)) < glass_share, 1, 0).astype(np.uint32) for s in build.slot]
    pts = np.concatenate(build.pts)
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    ground = Mesh()
    ground.grid((lo[0] - 50, lo[1] - 50, 0), (hi[0] - lo[0] + 100, 0, 0), (0, hi[1] - lo[1] + 100, 0), 40, 40)
    s = assemble([(build, True, True), (ground, False, True)])
    s["quad"] = q
    return s


def random_city(seed, n_boxes=40, extent=60.0, q=2.0, porous=False, glass=False, thin=False):
    """A small random box pile on a ground, every face a sensor; slots: 0 opaque, 1 porous, 2 glass, 3 thin pane box."""
    rng = np.random.default_rng(seed)
    build, ground, panes = Mesh(), Mesh(), Mesh()
    ground.grid((-extent, -extent, 0), (2 * extent, 0, 0), (0, 2 * extent, 0), 8, 8)
    for _ in range(n_boxes):
        x0, y0 = rng.uniform(-extent * 0.8, extent * 0.6, 2)
        w, d = rng.uniform(3, 15, 2)
        h = rng.uniform(3, 25)
        choices = [0, 0] + ([1] if porous else []) + ([2] if glass else [])
        _box_faces(build, x0, y0, w, d, h, q, int(rng.choice(choices)))
    if thin:   # 10 cm pane boxes (thin solids), slot 3
        for _ in range(6):
            x0, y0 = rng.uniform(-extent * 0.7, extent * 0.7, 2)
            _box_faces(panes, x0, y0, 8.0, 0.05, rng.uniform(4, 12), 4.0, 3)
    meshes = [(build, True, True), (ground, True, True)]
    if thin:
        meshes.append((panes, False, True))
    return assemble(meshes)


def hemisphere_dirs(n_sky, n_sun, seed=0):
    """A direction table shaped as the reference's: [sky n_sky | ground = -sky | sun n_sun], unit float32."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(0.02, 1.0, n_sky)
    a = rng.uniform(0, 2 * np.pi, n_sky)
    r = np.sqrt(1 - z * z)
    sky = np.stack([r * np.sin(a), r * np.cos(a), z], axis=1)
    z2 = rng.uniform(0.01, 0.95, n_sun)
    a2 = rng.uniform(0, 2 * np.pi, n_sun)
    r2 = np.sqrt(1 - z2 * z2)
    sun = np.stack([r2 * np.sin(a2), r2 * np.cos(a2), z2], axis=1)
    D = np.concatenate([sky, -sky, sun]).astype(np.float32)
    return D


def views_city(seed=42, n_buildings=20000, target_tris=2_000_000, n_sensors=50_000):
    """The views city: rotated boxes with gable roofs (14 triangles each) on a street grid, the facades of the first
    buildings remeshed into ~n_sensors receiver quads (mesh sizes vary from building to building), and three target
    groups - a water strip (label 3), park lawns (label 4) and a landmark tower (label 5) - on a ground of quads that
    brings the scene to ~target_tris triangles. Labels: 2 obstruction, 3.. targets (the reference's views classes)."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(np.sqrt(n_buildings * 1.15)))
    pitch = 40.0
    lots = [(i, j) for j in range(side) for i in range(side)]
    park_lots = set(rng.choice(len(lots), max(1, len(lots) // 12), replace=False).tolist())
    centre_lot = (side // 2) * side + side // 2
    park_lots.discard(centre_lot)
    V, T, L = [], [], []
    nv = 0

    def add(verts, tris, label):
        nonlocal nv
        V.append(np.asarray(verts, np.float64))
        T.append(np.asarray(tris, np.int64) + nv)
        L.append(np.full(len(tris), label, np.uint8))
        nv += len(verts)

    sens = Mesh()   # receivers: facade quads of the first buildings
    sens_target = n_sensors
    made = 0
    b = 0
    for k, (i, j) in enumerate(lots):
        x0, y0 = i * pitch, j * pitch
        if k in park_lots:
            add([(x0 + 2, y0 + 2, 0.05), (x0 + 38, y0 + 2, 0.05), (x0 + 38, y0 + 38, 0.05), (x0 + 2, y0 + 38, 0.05)], [(0, 1, 2), (0, 2, 3)], 4)
            continue
        if k == centre_lot:   # the landmark: a 30 x 30 m tower, 150 m
            c = [(x0 + 5, y0 + 5), (x0 + 35, y0 + 5), (x0 + 35, y0 + 35), (x0 + 5, y0 + 35)]
            vs = [(x, y, 0) for x, y in c] + [(x, y, 150) for x, y in c]
            add(vs, [(0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5), (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7), (4, 5, 6), (4, 6, 7)], 5)
            continue
        if b >= n_buildings:
            continue
        b += 1
        w, d = sorted(rng.uniform(10, 30, 2))[::-1]
        h = rng.uniform(8, 40)
        rh = rng.uniform(2, 6)
        th = rng.uniform(0, np.pi)
        cx, cy = x0 + 20, y0 + 20
        ct, st = np.cos(th), np.sin(th)
        loc = [(-w / 2, -d / 2), (w / 2, -d / 2), (w / 2, d / 2), (-w / 2, d / 2)]
        c = [(cx + ct * a - st * bb, cy + st * a + ct * bb) for a, bb in loc]
        r0 = (cx + ct * (-w / 2), cy + st * (-w / 2))
        r1 = (cx + ct * (w / 2), cy + st * (w / 2))
        roof = [(x, y, h) for x, y in c] + [(r0[0], r0[1], h + rh), (r1[0], r1[1], h + rh)]
        # roof: south slope c0 c1 R1 R0, north slope c2 c3 R0 R1, gables c3 c0 R0 and c1 c2 R1 (indices into roof)
        rt = [(0, 1, 5), (0, 5, 4), (2, 3, 4), (2, 4, 5), (3, 0, 4), (1, 2, 5)]
        if made < sens_target:   # facades as receivers, ~2.5 m quads
            for q in range(4):
                a0, a1 = c[q], c[(q + 1) % 4]
                L_ = np.hypot(a1[0] - a0[0], a1[1] - a0[1])
                nu, nvv = max(1, int(round(L_ / 2.5))), max(1, int(round(h / 2.5)))
                sens.grid((a0[0], a0[1], 0), (a1[0] - a0[0], a1[1] - a0[1], 0), (0, 0, h), nu, nvv)
                made += nu * nvv
            add(roof, rt, 2)
        else:
            vs = [(x, y, 0) for x, y in c] + roof
            wt = [(0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5), (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
            add(vs, wt + [(4 + a, 4 + bb, 4 + cc) for a, bb, cc in rt], 2)
    W = side * pitch
    add([(0, -60, 0.05), (W, -60, 0.05), (W, -10, 0.05), (0, -10, 0.05)], [(0, 1, 2), (0, 2, 3)], 3)   # water strip
    have = sum(len(t) for t in T) + 2 * sum(len(q) for q in sens.quads)
    G = max(1, int(np.sqrt(max(0, target_tris - have) / 2)))
    gm = Mesh()
    gm.grid((-100, -160, 0), (W + 200, 0, 0), (0, W + 260, 0), G, G)
    gp, gq, _ = gm.arrays()
    add(gp, np.concatenate([gq[:, [0, 1, 2]], gq[:, [0, 2, 3]]], axis=1).reshape(-1, 3), 2)
    # assemble: receivers first (they block too), then the context
    sp, sq, _ = sens.arrays()
    allv = np.concatenate([sp] + V)
    centre = 0.5 * (allv.min(axis=0) + allv.max(axis=0))
    st_tri = np.concatenate([sq[:, [0, 1, 2]], sq[:, [0, 2, 3]]], axis=1).reshape(-1, 3)
    v = np.concatenate([sp - centre] + [x - centre for x in V]).astype(np.float32)
    tri = np.concatenate([st_tri] + [t + len(sp) for t in T]).astype(np.uint32)
    label = np.concatenate([np.full(len(st_tri), 2, np.uint8)] + L)
    c_, n_ = _faces_geom(sp - centre, sq)
    return dict(v=v, tri=tri, label=label, P=c_.astype(np.float32), N=n_.astype(np.float32), groundZ=float(0 - centre[2]), centre=centre)


def views_grid(fov, cell, lo=-70.0, hi=50.0):
    """The reference's field (views.cpp:122-136): nAz x nEl cells, per row sin of its bottom / top elevation, row
    weights (solid angle, normalised so the field sums to 1)."""
    flat = lo == hi
    nAz = max(1, int(round(fov / cell)))
    nEl = 1 if flat else max(1, int(round((hi - lo) / cell)))
    dAz, dEl = fov / nAz, (hi - lo) / nEl
    rowSin = np.zeros((nEl, 2), np.float32)
    wRow = np.zeros(nEl)
    for k in range(nEl):
        top, bot = np.sin(np.radians(hi - k * dEl)), np.sin(np.radians(hi - (k + 1) * dEl))
        rowSin[k] = (bot, top)
        wRow[k] = np.radians(dAz) * (1 if flat else top - bot)
    wRow /= wRow.sum() * nAz
    return nAz, nEl, float(dAz), rowSin, wRow


# ---------------------------------------------------------------------------------------------- sky of the urban year
KRF, KGF, KBF = 0.265074126, 0.670114631, 0.064811243   # Radiance CIE_rf / gf / bf (bright())


def patch_dirs(mf):
    """Reinhart / Tregenza patch centres (gendaymtx order, src/sky.cpp:240-270) and their solid angles, float as the
    reference's make_patches + dir_from_altaz."""
    tnaz = [30, 30, 24, 24, 18, 12, 6]
    alpha = (np.pi / 2) / (7 * mf + .5)
    alt, azi, om = [], [], []
    for i in range(7 * mf):
        n = tnaz[i // mf] * mf
        for j in range(n):
            alt.append(np.float32(alpha * (i + .5)))
            azi.append(np.float32(2 * np.pi * j / n))
            om.append(np.float32(2 * np.pi * (np.sin(alpha * (i + 1)) - np.sin(alpha * i)) / n))
    alt.append(np.float32(np.pi / 2)); azi.append(np.float32(0)); om.append(np.float32(2 * np.pi * (1 - np.cos(alpha * .5))))
    a, z = np.array(alt, np.float64), np.array(azi, np.float64)
    D = np.stack([np.cos(a) * np.sin(z), np.cos(a) * np.cos(z), np.sin(a)], axis=1).astype(np.float32)
    return D, np.array(om, np.float32)


def urban_year_sky(e, mf, weather):
    """The urban weather year's series operands built on the GPU: NOAA sun per hour (kgb_sun_noaa) and the Perez sky per
    hour and patch (kgb_sky, FP64), as the reference's run.cpp builds them on the host (src/run.cpp:350-419, physical
    mode, radiometric). weather: [2 x 8760] DNI and DHI of the year (Berlin, UTC+1). Returns the series inputs of the
    non-night hours: S [P x T], g [T], Sdc [(P + 1) x T] (bin 0 the ground, bin 1 + p the patch radiance plus the binned
    sun), the sun-up hours' directions, columns and DNI, and the build's wall time."""
    import time
    w = np.asarray(weather, np.float64)
    dim = [31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31]
    month = np.repeat(np.arange(1, 13), [24 * d for d in dim])
    day = np.concatenate([np.repeat(np.arange(1, d + 1), 24) for d in dim])
    hour = np.tile(np.arange(24) + 0.5, 365)
    jd = np.repeat(np.arange(1, 366), 24)
    rows = np.stack([np.full(8760, 52.52), np.full(8760, 13.41), np.full(8760, 1.0), month, day, hour, np.zeros(8760)], axis=1)
    t0 = time.perf_counter()
    sun = e.sun_noaa(rows)
    steps = np.stack([jd, np.radians(sun[:, 0]), np.radians(sun[:, 1]), w[0], w[1]], axis=1)
    sky = e.sky(mf, steps, grefl=0.2, sun=False, sky=True, visible=False)
    sunbin = e.sky(mf, steps, grefl=0.2, sun=True, sky=False, visible=False)   # the sun as gendaymtx bins it (AddDirect)
    sky_s = time.perf_counter() - t0
    bright = KRF * sky[:, :, 0] + KGF * sky[:, :, 1] + KBF * sky[:, :, 2]
    bright_sun = KRF * sunbin[:, :, 0] + KGF * sunbin[:, :, 1] + KBF * sunbin[:, :, 2]
    col = (w[0] + w[1]) > 1e-4
    colOf = np.cumsum(col) - 1
    S = np.ascontiguousarray(bright[col, 1:].T, np.float32)
    g = np.ascontiguousarray(bright[col, 0], np.float32)
    Sdc = np.concatenate([g[None, :], (S.astype(np.float64) + bright_sun[col, 1:].T).astype(np.float32)]).astype(np.float32)
    up = sun[:, 2] > 0
    sunVec = sun[up, 3:6].astype(np.float32)
    ups = np.nonzero(up)[0]
    sunStep = np.where(col[ups], colOf[ups], 0).astype(np.int32)
    sunW = np.where(col[ups], w[0][ups], 0).astype(np.float32)
    return dict(S=S, g=g, Sdc=Sdc, sunVec=sunVec, sunStep=sunStep, sunW=sunW, sky_s=sky_s, T=int(col.sum()))
