"""A plain-Python model of the seam kernels' formulation (leven_gb300/csrc/
lvn_seam.cu), used by the CPU tests to check that formulation against the
oracle's literal restatement of the reference's recursion
(Octree_ConstructUpwards + ContourCellProc, octree.cpp:90-474):

* leaves numbered in the Morton order of their minimum corners;
* one quad per final edge segment, found from the smallest leaf's edges with
  the three other leaves looked up by region;
* the recursion's order restored by sorting on the recursion path.

Test infrastructure only; small inputs."""
import bisect

CLIPMAP_LEAF_SIZE = 256
EDGE_VMAP = [(0, 4), (1, 5), (2, 6), (3, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 1), (2, 3), (4, 5), (6, 7)]
CELL_FACE = [(0, 4, 0), (1, 5, 0), (2, 6, 0), (3, 7, 0), (0, 2, 1), (4, 6, 1), (1, 3, 1), (5, 7, 1), (0, 1, 2),
             (2, 3, 2), (4, 5, 2), (6, 7, 2)]
CELL_EDGE = [(0, 1, 2, 3, 0), (4, 5, 6, 7, 0), (0, 4, 1, 5, 1), (2, 6, 3, 7, 1), (0, 2, 4, 6, 2), (1, 3, 5, 7, 2)]
FACE_FACE = [[(4, 0, 0), (5, 1, 0), (6, 2, 0), (7, 3, 0)], [(2, 0, 1), (6, 4, 1), (3, 1, 1), (7, 5, 1)],
             [(1, 0, 2), (3, 2, 2), (5, 4, 2), (7, 6, 2)]]
FACE_EDGE = [[(1, 4, 0, 5, 1, 1), (1, 6, 2, 7, 3, 1), (0, 4, 6, 0, 2, 2), (0, 5, 7, 1, 3, 2)],
             [(0, 2, 3, 0, 1, 0), (0, 6, 7, 4, 5, 0), (1, 2, 0, 6, 4, 2), (1, 3, 1, 7, 5, 2)],
             [(1, 1, 0, 3, 2, 0), (1, 5, 4, 7, 6, 0), (0, 1, 5, 0, 4, 1), (0, 3, 7, 2, 6, 1)]]
PROCESS_EDGE = [(3, 2, 1, 0), (7, 5, 6, 4), (11, 10, 9, 8)]


def cbit(c, a):
    return (c >> (2 - a)) & 1


def morton(p, lev):
    code = 0
    for bit in range(lev - 1, -1, -1):
        code = (code << 3) | (((p[0] >> bit) & 1) << 2) | (((p[1] >> bit) & 1) << 1) | ((p[2] >> bit) & 1)
    return code


def path_key(root, d, line, t0, ln):
    digits = []
    a1, a2 = [a for a in range(3) if a != d]
    m, S = [0, 0, 0], root
    while True:
        h = S // 2
        mid = [m[a] + h for a in range(3)]
        on1, on2, hd = line[a1] == mid[a1], line[a2] == mid[a2], int(t0 >= mid[d])
        if not on1 and not on2:
            c = (hd << (2 - d)) | (int(line[a1] > mid[a1]) << (2 - a1)) | (int(line[a2] > mid[a2]) << (2 - a2))
            digits.append((c, 5))
            m = [m[a] + cbit(c, a) * h for a in range(3)]
            S = h
            continue
        if on1 and on2:
            e = [i for i in range(6) if CELL_EDGE[i][4] == d and cbit(CELL_EDGE[i][0], d) == hd][0]
            digits.append((20 + e, 5))
            e0, es = m[d] + hd * h, h
            break
        a, b = (a1, a2) if on1 else (a2, a1)
        bs = int(line[b] > mid[b])
        c0 = (bs << (2 - b)) | (hd << (2 - d))
        c1 = c0 | (1 << (2 - a))
        f = [i for i in range(12) if CELL_FACE[i][0] == c0 and CELL_FACE[i][1] == c1][0]
        digits.append((8 + f, 5))
        fb, fd, fs = m[b] + bs * h, m[d] + hd * h, h
        while True:
            hh = fs // 2
            fhd = int(t0 >= fd + hh)
            if line[b] != fb + hh:
                fbs = int(line[b] > fb + hh)
                i4 = [i for i in range(4) if cbit(FACE_FACE[a][i][1], b) == fbs and cbit(FACE_FACE[a][i][1], d) == fhd][0]
                digits.append((i4, 3))
                fb, fd, fs = fb + fbs * hh, fd + fhd * hh, hh
                continue
            i4 = [i for i in range(4) if FACE_EDGE[a][i][5] == d and cbit(FACE_EDGE[a][i][1], d) == fhd][0]
            digits.append((4 + i4, 3))
            e0, es = fd + fhd * hh, hh
            break
        break
    while es > ln:
        eh = es // 2
        hf = int(t0 >= e0 + eh)
        digits.append((hf, 1))
        e0, es = e0 + hf * eh, eh
    key, nbits = 0, 0
    for v, w in digits:
        nbits += w
        key |= v << (64 - nbits)
    assert nbits <= 64
    return key


def contour(host_min, host_size, leaves):
    """leaves: list of (min xyz absolute, size, corners).  Returns (order,
    triangles): order = the leaves' indices in vertex order, triangles as
    vertex-rank triples in the recursion's order."""
    root = 2 * host_size
    unit = min(s for _, s, _ in leaves)
    lev = (root // unit).bit_length() - 1
    rel = [tuple(m[a] - host_min[a] for a in range(3)) for m, _, _ in leaves]
    keyed = sorted(range(len(leaves)), key=lambda i: morton([r // unit for r in rel[i]], lev))
    codes = [morton([r // unit for r in rel[i]], lev) for i in keyed]
    sizes = [leaves[i][1] for i in keyed]

    def find(rmin, s):
        if any(r < 0 or r >= root for r in rmin):
            return -1
        k = morton([r // unit for r in rmin], lev)
        vol = (s // unit) ** 3
        lo = bisect.bisect_left(codes, k)
        if lo < len(codes) and codes[lo] < k + vol:
            return lo if codes[lo] == k and sizes[lo] >= s else -2
        if lo > 0 and sizes[lo - 1] > s:
            sl = (sizes[lo - 1] // unit).bit_length() - 1
            if k >> (3 * sl) == codes[lo - 1] >> (3 * sl):
                return lo - 1
        return -1

    quads = []
    for r, i in enumerate(keyed):
        lmin, s, corners = rel[i], leaves[i][1], leaves[i][2]
        for e in range(12):
            c0, c1 = EDGE_VMAP[e]
            m0, m1 = (corners >> c0) & 1, (corners >> c1) & 1
            if m0 == m1:
                continue
            d = e >> 2
            j = PROCESS_EDGE[d].index(e)
            line = [lmin[a] + cbit(c0, a) * s for a in range(3)]
            ranks = []
            for q in range(4):
                if q == j:
                    ranks.append(r)
                    continue
                child = CELL_EDGE[2 * d][q]
                ranks.append(find([lmin[a] if a == d else line[a] - s + cbit(child, a) * s for a in range(3)], s))
            if min(ranks) < 0:
                continue
            qs = [sizes[x] for x in ranks]
            if qs.index(min(qs)) != j:
                continue
            blocks = {tuple((rel[keyed[x]][a] + host_min[a]) & ~(CLIPMAP_LEAF_SIZE - 1) for a in range(3))
                      for x in ranks}
            if len(blocks) == 1:
                continue
            quads.append((path_key(root, d, line, lmin[d], s), ranks, m1 != 1))
    quads.sort()
    tris = []
    for _, (i0, i1, i2, i3), flip in quads:
        tris += [(i0, i3, i1), (i0, i2, i3)] if flip else [(i0, i1, i3), (i0, i3, i2)]
    return keyed, tris


def in_root(mn, size, root_min, root_size):
    return all(0 <= mn[a] - root_min[a] and mn[a] - root_min[a] + size <= root_size and
               (mn[a] - root_min[a]) % size == 0 for a in range(3))


def find_active(mn, size, active, root_min, root_size):
    """FindActiveNodes (clipmap.cpp:1449-1472) over the complete octree."""
    out = []

    def inside(bmin, bsize, p):
        return all(bmin[a] <= p[a] < bmin[a] + bsize for a in range(3))

    def visit(nmin, nsize):
        if inside(nmin, nsize, mn) or inside(mn, size, nmin):
            if (tuple(nmin), nsize) in active:
                out.append(active[(tuple(nmin), nsize)])
            elif nsize > CLIPMAP_LEAF_SIZE:
                h = nsize // 2
                for i in range(8):
                    visit([nmin[0] + ((i >> 2) & 1) * h, nmin[1] + ((i >> 1) & 1) * h, nmin[2] + (i & 1) * h], h)

    visit(list(root_min), root_size)
    return out


def filter_seam_node(i, b, mn, mx):
    return [mx[0] == b[0] or mx[1] == b[1] or mx[2] == b[2], mn[2] == b[2], mn[1] == b[1],
            mn[1] == b[1] or mn[2] == b[2], mn[0] == b[0], mn[0] == b[0] or mn[2] == b[2],
            mn[0] == b[0] or mn[1] == b[1], tuple(mn) == tuple(b)][i]


def gather(chunks, offsets, seams, vpc, root_min, root_size, h):
    """SelectSeamNodes over the active nodes around host h: list of (min,
    size, corners, seam row), each node once."""
    active = {(tuple(mn), s): c for c, (mn, s) in enumerate(chunks)}
    hmin, hs = chunks[h]
    bounds = [hmin[a] + hs for a in range(3)]
    got = {}
    for i in range(8):
        nmin = [hmin[0] + ((i >> 2) & 1) * hs, hmin[1] + ((i >> 1) & 1) * hs, hmin[2] + (i & 1) * hs]
        if not in_root(nmin, hs, root_min, root_size):
            continue
        for c in find_active(nmin, hs, active, root_min, root_size):
            cmin, cs = chunks[c]
            ns, ext = cs // vpc, (cs // (vpc * 4)) * 4
            for k in range(offsets[c], offsets[c + 1]):
                row = seams[k]
                mn = [int(row[a]) * ns + cmin[a] for a in range(3)]
                mx = [mn[a] + ext for a in range(3)]
                if not all(hmin[a] <= mn[a] < hmin[a] + 2 * hs for a in range(3)):
                    continue
                if filter_seam_node(i, bounds, mn, mx):
                    got[tuple(mn)] = (tuple(mn), ns, int(row[3]) & 0xFF, k)
    return list(got.values())
