"""Seeded synthetic workloads for the chunk-meshing path.

Chunk lists are world-space (min, size) pairs as the engine passes them to
generateChunkMesh (1 voxel = 4 world units at LOD0, a 64^3 chunk at LOD k has
size 256 * 2^k).  CSG operations are in density units, as
Clipmap::queueCSGOperation produces them (leven/src/clipmap.cpp:1618-1636).

Random numbers come from a 32-bit Mersenne twister with std::mt19937's
seeding, so the same seed gives the same operations in C++ and Python;
floats are (x >> 8) * 2^-24, uniform in [0, 1).
"""
from dataclasses import dataclass

MATERIAL_AIR = 201


class MT19937:
    """std::mt19937 (seed_seq-free constructor semantics)."""

    def __init__(self, seed=5489):
        self.mt = [0] * 624
        self.mt[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            self.mt[i] = (1812433253 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self.index = 624

    def _twist(self):
        mt = self.mt
        for i in range(624):
            y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
            v = mt[(i + 397) % 624] ^ (y >> 1)
            if y & 1:
                v ^= 0x9908B0DF
            mt[i] = v
        self.index = 0

    def u32(self):
        if self.index >= 624:
            self._twist()
        y = self.mt[self.index]
        self.index += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def uniform(self, lo, hi):
        return lo + (hi - lo) * ((self.u32() >> 8) * (1.0 / 16777216.0))


@dataclass
class Op:
    type: int          # 0 add (union), 1 subtract
    brush_shape: int   # 0 cube, 1 sphere
    material: int
    origin: tuple      # density units
    dimensions: tuple  # half extents / radius in [0]
    rotate_y: float = 0.0

    def as_tuple(self):
        return (self.type, self.brush_shape, self.material, self.rotate_y, self.origin, self.dimensions)


@dataclass
class Workload:
    name: str
    chunks: list       # [((x, y, z), size)]
    ops: list          # [Op]
    density: dict      # keyword arguments of leven_gb300.set_density
    noise_seed: int = 1
    voxels_per_chunk: int = 64


FBM2D = dict(mode=1, octaves2=8, freq2=1.0 / 256.0, lacunarity2=2.0, gain2=0.5, amp2=48.0)
CAVES = dict(mode=2, octaves2=8, freq2=1.0 / 256.0, lacunarity2=2.0, gain2=0.5, amp2=48.0,
             octaves3=6, freq3=1.0 / 64.0, lacunarity3=2.0, gain3=0.5, amp3=12.0)


def plain_one_chunk():
    """One LOD0 64^3 chunk, density-space origin (0, 32, 0), 2D fBm terrain
    (8 octaves, 1/256, lacunarity 2, gain 0.5, amplitude 48), seed 1."""
    return Workload("plain-one-chunk-64", [((0, 128, 0), 256)], [], FBM2D)


def csg_ops(n, seed, region_lo, region_hi, rmin=2.0, rmax=12.0):
    """n operations, half sphere-subtract (type 1, sphere, AIR) and half
    box-union (type 0, cube, material 1), centres uniform in the region,
    radius / half extents uniform in [rmin, rmax] voxels, no rotation."""
    rng = MT19937(seed)
    ops = []
    for _ in range(n):
        subtract = (rng.u32() & 1) == 1
        c = tuple(rng.uniform(region_lo[i], region_hi[i]) for i in range(3))
        if subtract:
            r = rng.uniform(rmin, rmax)
            ops.append(Op(1, 1, MATERIAL_AIR, c, (r, r, r)))
        else:
            ops.append(Op(0, 0, 1, c, tuple(rng.uniform(rmin, rmax) for _ in range(3))))
    return ops


def tiled_csg(nx=8, ny=2, nz=8, n_ops=32, seed=1):
    """LOD0 64^3 chunks tiling a (64 nx) x (64 ny) x (64 nz) voxel region,
    y centred on 0 so that the fBm surface is inside, with n_ops seeded CSG
    operations.  The default is 8 x 2 x 8 = 128 chunks over 512 x 128 x 512
    voxels and 32 operations."""
    y0 = -(64 * ny) // 2
    chunks = [((256 * i, 4 * y0 + 256 * j, 256 * k), 256) for k in range(nz) for j in range(ny) for i in range(nx)]
    ops = csg_ops(n_ops, seed, (0.0, float(y0), 0.0), (64.0 * nx, float(y0 + 64 * ny), 64.0 * nz))
    return Workload(f"tiled-csg-{len(chunks)}x64^3-{n_ops}ops", chunks, ops, FBM2D)


def op_bounds(op):
    """CalcCSGOperationBounds (clipmap.cpp:1638-1643)."""
    import numpy as np

    lo, hi = [], []
    for i in range(3):
        half = int(np.float32(op.dimensions[i]) * np.float32(4.0)) + 2
        origin = int((np.float32(op.origin[i]) - np.float32(0.5)) * np.float32(4.0))
        lo.append(origin - half)
        hi.append(origin + half)
    return lo, hi


def ops_for_chunk(ops, mn, size):
    """Stored operations whose AABB overlaps the chunk (compute_density_field.cpp:255-263)."""
    out = []
    for op in ops:
        lo, hi = op_bounds(op)
        if not (mn[0] + size < lo[0] or mn[1] + size < lo[1] or mn[2] + size < lo[2] or mn[0] > hi[0] or
                mn[1] > hi[1] or mn[2] > hi[2]):
            out.append(op)
    return out


# Clipmap LOD selection (leven/src/clipmap.cpp:28-41, 1056-1128)
CLIPMAP_LEAF_SIZE = 256
NUM_LODS = 6
LOD_MAX_NODE_SIZE = CLIPMAP_LEAF_SIZE * (1 << (NUM_LODS - 1))
LOD_ACTIVE_DISTANCES = [0.0, CLIPMAP_LEAF_SIZE * 1.5, CLIPMAP_LEAF_SIZE * 3.5, CLIPMAP_LEAF_SIZE * 5.5,
                        CLIPMAP_LEAF_SIZE * 7.5, CLIPMAP_LEAF_SIZE * 13.5]


def distance_to_node(mn, size, cam):
    """DistanceToNode (clipmap.cpp:1056-1064): distance from the camera to the node's box."""
    d2 = 0.0
    for i in range(3):
        lo, hi = mn[i], mn[i] + size
        d = max(lo - cam[i], 0.0, cam[i] - hi)
        d2 += d * d
    return d2 ** 0.5


def select_clipmap_nodes(root_min, root_size, cam):
    """SelectActiveClipmapNodes (clipmap.cpp:1084-1128) over a complete clipmap
    octree whose leaves are CLIPMAP_LEAF_SIZE nodes: a node no larger than
    LOD_MAX_NODE_SIZE is selected when its distance to the camera is at least
    its LOD's active distance and no ancestor was selected."""
    out = []

    def visit(mn, size, parent_active):
        active = False
        if not parent_active and size <= LOD_MAX_NODE_SIZE:
            lod = (size // CLIPMAP_LEAF_SIZE).bit_length() - 1
            if distance_to_node(mn, size, cam) >= LOD_ACTIVE_DISTANCES[lod]:
                out.append((tuple(mn), size))
                active = True
        if size == CLIPMAP_LEAF_SIZE or parent_active or active:
            return  # nothing below a selected node is selected
        half = size // 2
        for i in range(8):
            off = ((i >> 2) & 1, (i >> 1) & 1, i & 1)  # CHILD_MIN_OFFSETS order
            visit(tuple(mn[k] + off[k] * half for k in range(3)), half, parent_active or active)

    visit(tuple(root_min), root_size, False)
    return out


CLIPMAP_ROOT_MIN = (-(1 << 14), -(1 << 14), -(1 << 14))
CLIPMAP_ROOT_SIZE = 1 << 15


def clipmap_cameras(n_paths=64, per_path=64, seed=1):
    """Camera positions for the clipmap selection workload: n_paths seeded
    straight paths of per_path positions each through the 2^15-unit world
    centred on the origin, as the engine re-selects while the camera travels
    (start x, z U[-2048, 2048], y U[-64, 64]; 256 * U[-1, 1] per step in x and
    z); float32, (n_paths * per_path, 3)."""
    import numpy as np

    rng = MT19937(seed)
    out = []
    for _ in range(n_paths):
        cam0 = (rng.uniform(-2048.0, 2048.0), rng.uniform(-64.0, 64.0), rng.uniform(-2048.0, 2048.0))
        step = (rng.uniform(-1.0, 1.0) * 256.0, 0.0, rng.uniform(-1.0, 1.0) * 256.0)
        out += [[cam0[i] + k * step[i] for i in range(3)] for k in range(per_path)]
    return np.array(out, np.float32)


def clipmap_frame(seed=1):
    """The clipmap's active nodes for one camera: SelectActiveClipmapNodes over
    the 2^15-unit world at the starting camera of the caves path (428 nodes,
    LOD 0-5, a disjoint tiling of the world), caves density."""
    rng = MT19937(seed)
    cam = (rng.uniform(-2048.0, 2048.0), rng.uniform(-64.0, 64.0), rng.uniform(-2048.0, 2048.0))
    nodes = select_clipmap_nodes(CLIPMAP_ROOT_MIN, CLIPMAP_ROOT_SIZE, cam)
    return Workload(f"clipmap-frame-{len(nodes)}chunks-lod0-5", [(tuple(mn), size) for mn, size in nodes], [], CAVES)


def clipmap_caves(n_chunks=1024, max_lod=4, seed=1):
    """n_chunks chunks over clipmap LODs 0..max_lod, density = 2D
    fBm heightfield + 3D fBm caves (6 octaves, 1/64, amplitude 12).  One
    camera selects about 370 nodes of LOD <= 4 (SelectActiveClipmapNodes over
    a 2^15-unit world centred on the origin), so the chunks are the union of
    the selections of a camera moving along a seeded straight path, as the
    engine re-meshes while the camera travels, nearest-first to the starting
    camera."""
    rng = MT19937(seed)
    cam0 = (rng.uniform(-2048.0, 2048.0), rng.uniform(-64.0, 64.0), rng.uniform(-2048.0, 2048.0))
    step = (rng.uniform(-1.0, 1.0) * 512.0, 0.0, rng.uniform(-1.0, 1.0) * 512.0)
    root_size = 1 << 15
    root_min = (-root_size // 2, -root_size // 2, -root_size // 2)
    chosen = {}
    for k in range(64):
        cam = tuple(cam0[i] + k * step[i] for i in range(3))
        for mn, size in select_clipmap_nodes(root_min, root_size, cam):
            if size <= CLIPMAP_LEAF_SIZE << max_lod:
                chosen[(mn, size)] = True
        if len(chosen) >= 2 * n_chunks:
            break
    nodes = sorted(chosen, key=lambda nd: (distance_to_node(nd[0], nd[1], cam0), nd[1], nd[0]))[:n_chunks]
    return Workload(f"clipmap-caves-{len(nodes)}chunks-lod0-{max_lod}", [(tuple(mn), size) for mn, size in nodes], [],
                    CAVES)


def clipmap_sweep(n_chunks=4096, max_lod=5, n_ops=64, seed=1):
    """The large clipmap sweep: n_chunks chunks over clipmap LODs 0..max_lod
    (voxel sizes 1-32), caves density (2D fBm heightfield + 3D fBm caves, as
    clipmap_caves), with n_ops seeded CSG operations stored and replayed per
    chunk through the plain path.

    Chunks: the union of SelectActiveClipmapNodes (2^15-unit world centred on
    the origin) over a camera moving along a seeded straight path in steps of
    256 * U[-1, 1] world units in x and z, until at least n_chunks nodes are
    active, then the n_chunks nearest the starting camera.  Operations: as
    csg_ops (half sphere-subtract, half box-union, radii / half extents U[2, 12]
    voxels), centres uniform over the camera path's x / z box (density units,
    widened by 64 voxels) and y in [-48, 48], the terrain's height band."""
    rng = MT19937(seed)
    cam0 = (rng.uniform(-2048.0, 2048.0), rng.uniform(-64.0, 64.0), rng.uniform(-2048.0, 2048.0))
    step = (rng.uniform(-1.0, 1.0) * 256.0, 0.0, rng.uniform(-1.0, 1.0) * 256.0)
    root_size = 1 << 15
    root_min = (-root_size // 2, -root_size // 2, -root_size // 2)
    chosen = {}
    cams = []
    for k in range(1024):
        cam = tuple(cam0[i] + k * step[i] for i in range(3))
        cams.append(cam)
        for mn, size in select_clipmap_nodes(root_min, root_size, cam):
            if size <= CLIPMAP_LEAF_SIZE << max_lod:
                chosen[(mn, size)] = True
        if len(chosen) >= n_chunks:
            break
    nodes = sorted(chosen, key=lambda nd: (distance_to_node(nd[0], nd[1], cam0), nd[1], nd[0]))[:n_chunks]
    lo = [min(c[i] for c in cams) / 4.0 - 64.0 for i in (0, 2)]
    hi = [max(c[i] for c in cams) / 4.0 + 64.0 for i in (0, 2)]
    ops = csg_ops(n_ops, seed + 1000, (lo[0], -48.0, lo[1]), (hi[0], 48.0, hi[1]))
    return Workload(f"clipmap-sweep-{len(nodes)}chunks-lod0-{max_lod}-caves-{n_ops}ops",
                    [(tuple(mn), size) for mn, size in nodes], ops, CAVES)
