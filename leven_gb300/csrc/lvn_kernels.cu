// lvn_kernels.cu -- the sm_103a kernels of the chunk-meshing pipeline.
//
// A batch of chunks flows through these stages (one launch each, all on one
// stream, no host round trip):
//
//   field      density per corner of each 66^3 field (heightfield modes reuse
//              the height term down each y column)      density_field.cl:11-37
//   csg        stored brush operations applied to the corner materials
//                                                       apply_csg_operation.cl:179-241
//   edge_*     count / plan / scatter of active field edges in the reference's
//              (hermite index, axis) order; plain edges touched by CSG are
//              dropped and CSG-created edges appended     density_field.cl:41-92,
//                                                       apply_csg_operation.cl:253-437
//   hermite    17-sample zero crossing + central-difference normal per edge
//                                                       density_field.cl:96-151,
//                                                       apply_csg_operation.cl:443-477
//   vox_*      count / plan / scatter of active voxels (leaf codes, edge
//              masks, dominant material)                octree.cl:142-223
//   hash_fill, edge_insert, node_insert
//              cuckoo tables, one per chunk and key set   cuckoo.cl:26-71
//   leaf       12 edge lookups, QEF accumulate + 10-sweep Jacobi solve,
//              MeshVertex written in place              octree.cl:236-331,475-487
//   mesh_*     quad emission with 3 node lookups per axis, seam nodes
//                                                       octree.cl:385-464,506-551
//
// Compactions are tile based: a CTA owns a tile of a chunk's dense domain,
// counts in one pass, and after a single-CTA plan kernel has scanned the tile
// counts it scatters with warp-shuffle block scans, which keeps the
// reference's linear-index order exactly.
#include "lvn_kernels.cuh"
#include "lvn_noise.cuh"

#include <cfloat>

namespace lvn {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kThreads = 256;
constexpr int kHermiteSmemThreads = 1024;   // k_hermite_smem: one CTA per SM
// batches at least this large take k_hermite_smem: with the caves density,
// whose 3D fBm reads the tables most, from 256 chunks (the sweep's first 256,
// 512 and 1024 chunks ran 5%, 4% and 4% faster a step than with k_hermite);
// with a heightfield alone from 2048 (a 128-chunk batch ran 8% slower)
constexpr int kHermiteSmemMinChunks = 2048;
constexpr int kHermiteSmemMinChunksCaves = 256;

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------

template <int VPC>
struct Geo {
    static constexpr int FD = VPC + 2;           // FIELD_DIM
    static constexpr int HD = VPC + 1;           // HERMITE_INDEX_SIZE
    static constexpr int F = FD * FD * FD;
    static constexpr int DEPTH = VPC == 8 ? 3 : VPC == 16 ? 4 : VPC == 32 ? 5 : 6;  // MAX_OCTREE_DEPTH
    static constexpr int SHIFT = DEPTH + 1;      // VOXEL_INDEX_SHIFT
    static constexpr int MASK = (1 << SHIFT) - 1;
    static constexpr int NBE = (FD * FD + kThreads - 1) / kThreads;   // field-row tiles
    static constexpr int NBV = (VPC * VPC + kThreads - 1) / kThreads; // voxel-row tiles
};

// EDGE_MAP / EDGE_VERTEX_MAP (shared_constants.cl:4-9, octree.cl:227-232) as
// nibble tables: {0,4},{1,5},{2,6},{3,7},{0,2},{1,3},{4,6},{5,7},{0,1},{2,3},{4,5},{6,7}
__device__ __forceinline__ int edge_c0(int i) { return (int)((0x642054103210ull >> (4 * i)) & 0xfull); }
__device__ __forceinline__ int edge_c1(int i) { return (int)((0x753176327654ull >> (4 * i)) & 0xfull); }

template <int VPC>
__device__ __forceinline__ uint32_t code_for_position(int x, int y, int z) {  // octree.cl:34-47
    uint32_t code = 1;
#pragma unroll
    for (int depth = Geo<VPC>::DEPTH - 1; depth >= 0; depth--) {
        const uint32_t c = (uint32_t)((((x >> depth) & 1) << 2) | (((y >> depth) & 1) << 1) | ((z >> depth) & 1));
        code = (code << 3) | c;
    }
    return code;
}

template <int VPC>
__device__ __forceinline__ void position_for_code(uint32_t code, int& x, int& y, int& z) {  // octree.cl:51-72
    x = y = z = 0;
#pragma unroll
    for (int i = 0; i < Geo<VPC>::DEPTH; i++) {
        const uint32_t c = code & 7u;
        code >>= 3;
        x |= (int)((c >> 2) & 1u) << i;
        y |= (int)((c >> 1) & 1u) << i;
        z |= (int)(c & 1u) << i;
    }
}

template <int VPC>
__device__ __forceinline__ int edge_key(int x, int y, int z, int axis) {
    return ((x | (y << Geo<VPC>::SHIFT) | (z << (2 * Geo<VPC>::SHIFT))) << 2) | axis;
}

// ---------------------------------------------------------------------------
// scans
// ---------------------------------------------------------------------------

__device__ __forceinline__ int warp_inclusive(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Exclusive scan over the CTA; `sm` holds NT/32 + 1 ints.  Safe to call
// back to back (ends with a barrier).
template <int NT>
__device__ __forceinline__ int block_exclusive(int v, int& total, int* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int inc = warp_inclusive(v);
    if (lane == 31) sm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int w = lane < NT / 32 ? sm[lane] : 0;
        const int wi = warp_inclusive(w);
        if (lane < NT / 32) sm[lane] = wi - w;
        if (lane == NT / 32 - 1) sm[NT / 32] = wi;
    }
    __syncthreads();
    const int r = inc - v + sm[warp];
    total = sm[NT / 32];
    __syncthreads();
    return r;
}

template <int NT>
__device__ __forceinline__ int block_sum(int v, int* sm) {
    int total;
    block_exclusive<NT>(v, total, sm);
    return total;
}

// Exclusive scan of `n` ints in place by one warp; returns the total.
__device__ __forceinline__ int warp_scan_array(int* a, int n) {
    const int lane = threadIdx.x & 31;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const int v = i < n ? a[i] : 0;
        const int inc = warp_inclusive(v);
        if (i < n) a[i] = carry + inc - v;
        carry += __shfl_sync(FULL, inc, 31);
    }
    return carry;
}

// Exclusive scan over n values held in global memory by one 1024-thread CTA.
// val(i) supplies the value; out(i, excl) receives the result.  Returns the total.
template <typename Val, typename Out>
__device__ __forceinline__ long long cta_scan(int n, Val val, Out out, long long* sm_carry, int* sm) {
    long long carry = 0;
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < n ? val(i) : 0;
        int total;
        const int ex = block_exclusive<1024>(v, total, sm);
        if (i < n) out(i, carry + ex);
        carry += total;
    }
    (void)sm_carry;
    return carry;
}

// ---------------------------------------------------------------------------
// IsPrime (primes.cpp:9-28)
// ---------------------------------------------------------------------------

__device__ bool is_prime_d(int x) {
    int o = 4, i = 5;
    for (;;) {
        const int q = x / i;
        if (q < i) return true;
        if (x == q * i) return false;
        o ^= 6;
        i += o;
    }
}


// ---------------------------------------------------------------------------
// cuckoo hash (cuckoo.cl:1-105)
// ---------------------------------------------------------------------------

// ((a * key mod 2^32) + b) mod 4294967291 mod m (cuckoo.cl:18-24).  h + b is
// below 2 * 4294967291, so the first remainder is one conditional subtract;
// the second uses magic = floor((2^32 - 1) / m), whose quotient estimate is
// at most two below the true quotient.
__device__ __forceinline__ uint32_t cuckoo_hash(uint32_t key, uint32_t a, uint32_t b, uint32_t mod, uint32_t magic) {
    unsigned long long s = (unsigned long long)(uint32_t)(a * key) + b;
    if (s >= 4294967291ull) s -= 4294967291ull;
    const uint32_t x = (uint32_t)s;
    uint32_t r = x - __umulhi(x, magic) * mod;
    if (r >= mod) r -= mod;
    if (r >= mod) r -= mod;
    return r;
}
__device__ __forceinline__ uint32_t stash_hash(uint32_t key, uint32_t a, uint32_t b) {
    unsigned long long s = (unsigned long long)(uint32_t)(a * key) + b;
    if (s >= 4294967291ull) s -= 4294967291ull;
    return (uint32_t)s % (uint32_t)CUCKOO_STASH_SIZE;
}

struct HashView {
    const unsigned long long* table;
    const unsigned long long* stash;
    uint32_t prime;
    uint32_t magic;
    int stash_used;
    uint32_t p[10];

    // Cuckoo_Find (cuckoo.cl:73-104); the stash probe reads the stash
    // All four probes are issued before any is tested: a key occupies at most
    // one slot, so testing them in order gives the sequential probe's answer.
    __device__ __forceinline__ uint32_t find(uint32_t key) const {
        unsigned long long e[CUCKOO_STASH_HASH_INDEX];
#pragma unroll
        for (int i = 0; i < CUCKOO_STASH_HASH_INDEX; i++) e[i] = table[cuckoo_hash(key, p[2 * i], p[2 * i + 1], prime, magic)];
#pragma unroll
        for (int i = 0; i < CUCKOO_STASH_HASH_INDEX; i++)
            if ((uint32_t)e[i] == key) return (uint32_t)(e[i] >> 32);
        if (stash_used) {
            const unsigned long long e = stash[stash_hash(key, p[8], p[9])];
            if ((uint32_t)e == key) return (uint32_t)(e >> 32);
        }
        return ~0u;
    }
};

// Cuckoo_InsertKeys (cuckoo.cl:26-71) for one key.  Returns 0 on success,
// 1 when the key went to the stash, -1 when the stash slot was taken.
__device__ __forceinline__ int cuckoo_insert(unsigned long long* table, unsigned long long* stash, uint32_t prime,
                                             uint32_t magic, const uint32_t* p, uint32_t key, uint32_t value) {
    unsigned long long entry = ((unsigned long long)value << 32) | key;
    uint32_t h = cuckoo_hash(key, p[0], p[1], prime, magic);
    for (int i = 0; i < CUCKOO_MAX_ITERATIONS; i++) {
        entry = atomicExch(&table[h], entry);
        if (entry == CUCKOO_EMPTY) return 0;
        key = (uint32_t)entry;
        const uint32_t h0 = cuckoo_hash(key, p[0], p[1], prime, magic);
        const uint32_t h1 = cuckoo_hash(key, p[2], p[3], prime, magic);
        const uint32_t h2 = cuckoo_hash(key, p[4], p[5], prime, magic);
        const uint32_t h3 = cuckoo_hash(key, p[6], p[7], prime, magic);
        if (h == h0) h = h1;
        else if (h == h1) h = h2;
        else if (h == h2) h = h3;
        else if (h == h3) h = h0;
    }
    key = (uint32_t)entry;
    const uint32_t hs = stash_hash(key, p[8], p[9]);
    const unsigned long long prev = atomicCAS(&stash[hs], CUCKOO_EMPTY, entry);
    return prev == CUCKOO_EMPTY ? 1 : -1;
}

// ---------------------------------------------------------------------------
// QEF (qef.cl), identical operation order to the restatement
// ---------------------------------------------------------------------------

struct Qef {
    float ata[6];
    float atb[3];
    float mp[4];
};

__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, float bx, float by, float bz, float bw) {
    return fmaf(aw, bw, fmaf(az, bz, fmaf(ay, by, ax * bx)));
}

__device__ __forceinline__ void givens_coeffs_sym(float a_pp, float a_pq, float a_qq, float& c, float& s) {
    if (a_pq == 0.f) { c = 1.f; s = 0.f; return; }
    const float tau = (a_qq - a_pp) / (2.f * a_pq);
    const float stt = sqrtf(1.f + tau * tau);
    const float tn = 1.f / ((tau >= 0.f) ? (tau + stt) : (tau - stt));
    c = 1.f / sqrtf(1.f + tn * tn);
    s = tn * c;
}

__device__ __forceinline__ void rot_xy(float& x, float& y, float c, float s) {
    const float u = x, v = y;
    x = c * u - s * v;
    y = s * u + c * v;
}

__device__ __forceinline__ void rotq_xy(float& x, float& y, float a, float c, float s) {
    const float cc = c * c, ss = s * s;
    const float mx = 2.f * c * s * a;
    const float u = x, v = y;
    x = cc * u - mx + ss * v;
    y = ss * u + mx + cc * v;
}

// svd_rotate (qef.cl:58-86) on the upper triangle vtav and V
template <int A, int B>
__device__ __forceinline__ void svd_rotate(float (&vt)[3][3], float (&v)[3][3]) {
    if (vt[A][B] == 0.f) return;
    float c, s;
    givens_coeffs_sym(vt[A][A], vt[A][B], vt[B][B], c, s);
    float x = vt[A][A], y = vt[B][B];
    rotq_xy(x, y, vt[A][B], c, s);
    vt[A][A] = x;
    vt[B][B] = y;
    x = vt[0][3 - B];
    y = vt[1 - A][2];
    rot_xy(x, y, c, s);
    vt[0][3 - B] = x;
    vt[1 - A][2] = y;
    vt[A][B] = 0.f;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        x = v[r][A];
        y = v[r][B];
        rot_xy(x, y, c, s);
        v[r][A] = x;
        v[r][B] = y;
    }
}

__device__ __forceinline__ float svd_invdet(float x, float tol) {
    return (fabsf(x) < tol || fabsf(1.f / x) < tol) ? 0.f : (1.f / x);
}

// qef_solve (qef.cl:239-256); returns the solved position (w = masspoint w)
__device__ __forceinline__ void qef_solve(const Qef& q, float& ox, float& oy, float& oz) {
    const float w = fmaxf(q.mp[3], 1.f);
    const float mx = q.mp[0] / w, my = q.mp[1] / w, mz = q.mp[2] / w, mw = q.mp[3] / w;
    const float* A = q.ata;
    float ax = dot4(A[0], A[1], A[2], 0.f, mx, my, mz, mw);
    float ay = A[1] * mx + A[3] * my + A[4] * mz;
    float az = A[2] * mx + A[4] * my + A[5] * mz;
    ax = q.atb[0] - ax;
    ay = q.atb[1] - ay;
    az = q.atb[2] - az;
    const float aw = 0.f - 0.f;
    float V[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
    float vt[3][3] = {{A[0], A[1], A[2]}, {0.f, A[3], A[4]}, {0.f, 0.f, A[5]}};
#pragma unroll 1
    for (int i = 0; i < 10; i++) {
        svd_rotate<0, 1>(vt, V);
        svd_rotate<0, 2>(vt, V);
        svd_rotate<1, 2>(vt, V);
    }
    const float d0 = svd_invdet(vt[0][0], 0.1f);
    const float d1 = svd_invdet(vt[1][1], 0.1f);
    const float d2 = svd_invdet(vt[2][2], 0.1f);
    float o[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) o[r][c] = V[r][0] * d0 * V[c][0] + V[r][1] * d1 * V[c][1] + V[r][2] * d2 * V[c][2];
    float x = dot4(o[0][0], o[0][1], o[0][2], 0.f, ax, ay, az, aw);
    float y = dot4(o[1][0], o[1][1], o[1][2], 0.f, ax, ay, az, aw);
    float z = dot4(o[2][0], o[2][1], o[2][2], 0.f, ax, ay, az, aw);
    ox = x + mx;
    oy = y + my;
    oz = z + mz;
}


// ---------------------------------------------------------------------------
// Octree simplification QEFs (not in the reference): a node's QEF in its own
// frame (origin at its min corner, unit = one voxel) with btb, so that the
// classic QEF value E(x) = x.ATA x - 2 x.ATb + btb is well conditioned.
// Children are summed in child order after moving them by d = child origin -
// node origin: ATb += ATA d, btb += 2 d.ATb + d.ATA d, mass point += w d.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void simp_zero(SimpQef& q) {
#pragma unroll
    for (int i = 0; i < 6; i++) q.ata[i] = 0.f;
    q.btb = q.w = q.pad[0] = q.pad[1] = q.pad[2] = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) q.atb[i] = q.mp[i] = q.ns[i] = 0.f;
}

// qef_add_point (qef.cl:170-191) plus btb, count and normal sum
__device__ __forceinline__ void simp_add_point(SimpQef& q, float px, float py, float pz, float nx, float ny, float nz) {
    q.ata[0] += nx * nx;
    q.ata[1] += nx * ny;
    q.ata[2] += nx * nz;
    q.ata[3] += ny * ny;
    q.ata[4] += ny * nz;
    q.ata[5] += nz * nz;
    const float bb = dot3(px, py, pz, nx, ny, nz);
    q.atb[0] += nx * bb;
    q.atb[1] += ny * bb;
    q.atb[2] += nz * bb;
    q.btb = fmaf(bb, bb, q.btb);
    q.mp[0] += px;
    q.mp[1] += py;
    q.mp[2] += pz;
    q.w += 1.f;
    q.ns[0] += nx;
    q.ns[1] += ny;
    q.ns[2] += nz;
}

__device__ __forceinline__ void simp_merge(SimpQef& q, const SimpQef& c, float dx, float dy, float dz) {
    const float* A = c.ata;
    const float adx = dot3(A[0], A[1], A[2], dx, dy, dz);
    const float ady = dot3(A[1], A[3], A[4], dx, dy, dz);
    const float adz = dot3(A[2], A[4], A[5], dx, dy, dz);
#pragma unroll
    for (int i = 0; i < 6; i++) q.ata[i] += A[i];
    q.atb[0] += c.atb[0] + adx;
    q.atb[1] += c.atb[1] + ady;
    q.atb[2] += c.atb[2] + adz;
    q.btb += c.btb + fmaf(2.f, dot3(dx, dy, dz, c.atb[0], c.atb[1], c.atb[2]), dot3(dx, dy, dz, adx, ady, adz));
    q.mp[0] += fmaf(c.w, dx, c.mp[0]);
    q.mp[1] += fmaf(c.w, dy, c.mp[1]);
    q.mp[2] += fmaf(c.w, dz, c.mp[2]);
    q.w += c.w;
    q.ns[0] += c.ns[0];
    q.ns[1] += c.ns[1];
    q.ns[2] += c.ns[2];
}

__device__ __forceinline__ float simp_error(const SimpQef& q, float x, float y, float z) {
    const float* A = q.ata;
    const float ax = dot3(A[0], A[1], A[2], x, y, z);
    const float ay = dot3(A[1], A[3], A[4], x, y, z);
    const float az = dot3(A[2], A[4], A[5], x, y, z);
    return fmaf(-2.f, dot3(x, y, z, q.atb[0], q.atb[1], q.atb[2]), dot3(x, y, z, ax, ay, az)) + q.btb;
}

// qef_solve on the node's QEF (its mass point is the running sum, which
// qef_solve divides by the count); a solution outside the node's cube of side
// s falls back to the mass point.  Returns the QEF value at the position.
__device__ __forceinline__ float simp_solve(const SimpQef& q, float s, float& ox, float& oy, float& oz) {
    Qef r;
#pragma unroll
    for (int i = 0; i < 6; i++) r.ata[i] = q.ata[i];
    r.atb[0] = q.atb[0];
    r.atb[1] = q.atb[1];
    r.atb[2] = q.atb[2];
    r.mp[0] = q.mp[0];
    r.mp[1] = q.mp[1];
    r.mp[2] = q.mp[2];
    r.mp[3] = q.w;
    float x, y, z;
    qef_solve(r, x, y, z);
    if (!(x >= 0.f && x <= s && y >= 0.f && y <= s && z >= 0.f && z <= s)) {
        x = q.mp[0] / q.w;
        y = q.mp[1] / q.w;
        z = q.mp[2] / q.w;
    }
    ox = x;
    oy = y;
    oz = z;
    return simp_error(q, x, y, z);
}

// ---------------------------------------------------------------------------
// stage 0: reset per-chunk state
// ---------------------------------------------------------------------------

__global__ void k_reset(BatchPtrs b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b.n) {
        ChunkState z;
        memset(&z, 0, sizeof(z));
        b.cs[i] = z;
    }
    if (i == 0) {
        BatchState z;
        memset(&z, 0, sizeof(z));
        *b.bs = z;
    }
}

// ---------------------------------------------------------------------------
// Field bit planes.  Row (y, z) of a chunk's field packs x = 0..65 into a
// uint4 (bits 0-31, 32-63, 64-65).  Plane 0: plain solid (material != AIR
// before CSG); plane 1: final air (material == AIR after CSG); plane 2:
// changed by this CSG batch.  Row index r = y + FD * z, so the linear
// successor of field point (FD-1, y, z) is bit 0 of row r + 1, as in the
// reference's linear field index.
// ---------------------------------------------------------------------------

template <int VPC>
__device__ __forceinline__ uint4* plane_ptr(const BatchPtrs& b, int c, int plane) {
    constexpr int R = (VPC + 2) * (VPC + 2);
    return b.planes + ((size_t)c * 3 + plane) * R;
}

// x + 1 neighbour: shift right by one bit across the row
__device__ __forceinline__ uint4 shr1(uint4 r) {
    return make_uint4((r.x >> 1) | (r.y << 31), (r.y >> 1) | (r.z << 31), (r.z >> 1) | (r.w << 31), r.w >> 1);
}
__device__ __forceinline__ uint4 and4(uint4 a, uint4 b) { return make_uint4(a.x & b.x, a.y & b.y, a.z & b.z, a.w & b.w); }
__device__ __forceinline__ uint4 or4(uint4 a, uint4 b) { return make_uint4(a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w); }
__device__ __forceinline__ uint4 xor4(uint4 a, uint4 b) { return make_uint4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w); }
__device__ __forceinline__ uint4 not4(uint4 a) { return make_uint4(~a.x, ~a.y, ~a.z, ~a.w); }
__device__ __forceinline__ int popc4(uint4 a) { return __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w); }
__device__ __forceinline__ bool bit4(uint4 a, int x) {
    const unsigned w = x < 32 ? a.x : x < 64 ? a.y : x < 96 ? a.z : a.w;
    return (w >> (x & 31)) & 1u;
}
// low `n` bits set (n <= 128)
__device__ __forceinline__ uint4 low_bits(int n) {
    auto m = [](int k) { return k <= 0 ? 0u : k >= 32 ? ~0u : ((1u << k) - 1u); };
    return make_uint4(m(n), m(n - 32), m(n - 64), m(n - 96));
}

// Height term and density for a density mode fixed at compile time, so a
// kernel carries one density's code (DensityFunc, noise.cl:225-268).
template <int MODE, class N>
__device__ __forceinline__ float height_m(const N& nz, const DensityParams& dp, float x, float z) {
    if (MODE == LVN_DENSITY_REFERENCE) return nz.terrain(x, z);
    return nz.fbm2(dp.octaves2, dp.freq2, dp.lacunarity2, dp.gain2, x, z);
}
template <int MODE, class N>
__device__ __forceinline__ float dens_h(const N& nz, const DensityParams& dp, float h, float x, float y, float z) {
    const float amp = MODE == LVN_DENSITY_REFERENCE ? 900.f : dp.amp2;  // MAX_TERRAIN_HEIGHT
    const float base = fmaf(-amp, h, y);
    if (MODE != LVN_DENSITY_CAVES) return base;
    return fmaf(dp.amp3, nz.fbm3(dp.octaves3, dp.freq3, dp.lacunarity3, dp.gain3, x, y, z), base);
}

// ---------------------------------------------------------------------------
// stage 1: density field (GenerateDefaultField, density_field.cl:11-37)
// One CTA per (z slice, chunk), one thread per x; heightfield modes evaluate
// the height term once per (x, z) column.  Writes the byte materials and the
// three bit planes (warp ballots along x).
// ---------------------------------------------------------------------------

template <int VPC, int MODE>
__global__ void __launch_bounds__(96) k_field(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ __align__(16) float sg[64];
    __shared__ uint32_t words[3][G::FD];  // solid-bit word of each warp, per row y
    stage_gradients(sg, b.grad);
    __syncthreads();
    const int c = blockIdx.y, z = blockIdx.x;
    if (b.s_on && b.sslot[c] >= 0) return;  // the surrogate's field (k_field_sdens)
    const int x = threadIdx.x;
    const bool valid = x < G::FD;
    // descriptor fields in registers: the byte stores below may alias them
    const int scale = b.desc[c].scale;
    const int ox = b.desc[c].off[0], oy = b.desc[c].off[1], oz = b.desc[c].off[2];
    const Noise nz{b.perm_t3, sg};
    const DensityParams& dp = b.density;
    const float wx = (float)(x * scale + ox);
    const float wz = (float)(z * scale + oz);
    const float h = valid ? height_m<MODE>(nz, dp, wx, wz) : 0.f;
    if (valid && b.hmap) b.hmap[(size_t)c * G::FD * G::FD + x + G::FD * z] = h;
    const int dm = b.default_material;
    const bool write_mats = b.need_mats != 0;
    uint8_t* mats = b.mats + (size_t)c * G::F + x + G::FD * G::FD * z;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    static_assert(MODE != LVN_DENSITY_CAVES, "a density with a 3D term uses k_field_caves");
    // y - amp * h rounds monotonically in y, so the column is solid below
    // the first y whose density is >= 0 and air from there up
    int ycross = 0;
    if (valid && dm != MATERIAL_AIR) {
        int lo = 0, hi = G::FD;  // first y in [lo, hi) with density >= 0, hi if none
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (dens_h<MODE>(nz, dp, h, wx, (float)(mid * scale + oy), wz) < 0.f) lo = mid + 1;
            else hi = mid;
        }
        ycross = lo;
    }
    if (valid && write_mats)
        for (int y = 0; y < G::FD; y++) mats[G::FD * y] = (uint8_t)(y < ycross ? dm : MATERIAL_AIR);
    // the warp's row words: every valid column is solid below the warp's
    // lowest crossing and air from its highest up, so only the rows between
    // need a ballot.  Lane l keeps rows l, l + 32 and l + 64.
    const unsigned vmask = __ballot_sync(FULL, valid);
    const int ymin = __reduce_min_sync(FULL, valid ? ycross : G::FD);
    const int ymax = __reduce_max_sync(FULL, valid ? ycross : 0);
    uint32_t w0 = 0, w1 = 0, w2 = 0;
    for (int y = ymin; y < ymax; y++) {
        const unsigned sb = __ballot_sync(FULL, y < ycross);
        if ((y & 31) == lane) {
            w0 = y < 32 ? sb : w0;
            w1 = y >= 32 && y < 64 ? sb : w1;
            w2 = y >= 64 ? sb : w2;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int y = lane + 32 * k;
        if (y < G::FD) words[warp][y] = y < ymin ? vmask : y >= ymax ? 0u : k == 0 ? w0 : k == 1 ? w1 : w2;
    }
    __syncthreads();
    // one thread per row writes the three 16-byte plane rows
    const uint4 V = low_bits(G::FD);
    uint4* P = plane_ptr<VPC>(b, c, 0) + G::FD * z;
    uint4* A = plane_ptr<VPC>(b, c, 1) + G::FD * z;
    uint4* X = plane_ptr<VPC>(b, c, 2) + G::FD * z;
    for (int y = threadIdx.x; y < G::FD; y += blockDim.x) {
        const uint4 p = make_uint4(words[0][y], words[1][y], words[2][y], 0u);
        P[y] = p;
        A[y] = and4(not4(p), V);
        X[y] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// ---------------------------------------------------------------------------
// stage 2: CSG materials (CSG_HermiteIndices + UpdateFieldMaterials,
// apply_csg_operation.cl:179-241) inside the chunk's operation bounding box;
// rows there get their final-air and changed bits rewritten.
// ---------------------------------------------------------------------------

// Field of a density with a 3D term (the cave fBm).  One CTA per z slice,
// one thread per x column.  The density is fma(amp3, fbm3, base) with
// base = y - amp2 h, and |amp3 fbm3| is at most b.cave_band, so where |base|
// exceeds it the sign of the density, which is all the field keeps, is the
// sign of base.  base rounds monotonically in y, so each column is solid below
// a first row ya (base < -band) and air from a first row yb (base > band),
// both found by bisection like the heightfield's crossing; only the rows
// [ya, yb) between them need the 3D term.  Those points go to a shared list
// that all lanes then evaluate, two octaves at a time, until the octaves left
// cannot change the sign; their solid bits are gathered into the row words
// with shared-memory atomics.
constexpr int kCaveBatch = 1024;  // listed points per batch of the stepped evaluation

template <int VPC>
__global__ void __launch_bounds__(96) k_field_caves(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ __align__(16) float sg[64];
    __shared__ float hs[G::FD];
    __shared__ uint32_t words[3][G::FD];
    __shared__ uint16_t list[G::FD * G::FD];
    __shared__ int wsum[3];
    __shared__ uint16_t bidx[2][kCaveBatch];  // the undecided points of a batch, ping-pong
    __shared__ float bnoise[2][kCaveBatch];   // their fBm partial sums
    __shared__ int bcount[2];
    stage_gradients(sg, b.grad);
    const int c = blockIdx.y, z = blockIdx.x;
    if (b.s_on && b.sslot[c] >= 0) return;  // the surrogate's field (k_field_sdens)
    const int scale = b.desc[c].scale;
    const int ox = b.desc[c].off[0], oy = b.desc[c].off[1], oz = b.desc[c].off[2];
    const DensityParams& dp = b.density;
    const float wz = (float)(z * scale + oz);
    __syncthreads();
    const Noise nz{b.perm_t3, sg};
    const int x = threadIdx.x;
    const bool valid = x < G::FD;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int dm = b.default_material;
    const float amp2 = dp.amp2, band = b.cave_band;
    const float h = valid ? height_m<LVN_DENSITY_CAVES>(nz, dp, (float)(x * scale + ox), wz) : 0.f;
    if (valid) {
        hs[x] = h;
        if (b.hmap) b.hmap[(size_t)c * G::FD * G::FD + x + G::FD * z] = h;
    }
    // ya: the first row whose base is not below -band; yb: the first row from
    // ya up whose base is above band (G::FD where there is none).  A NaN base
    // or band decides nothing: ya = 0, yb = G::FD, every row evaluated.  An AIR
    // default material makes every point air: no rows at all.
    int ya = 0, yb = 0;
    if (valid && dm != MATERIAL_AIR) {
        int lo = 0, hi = G::FD;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (fmaf(-amp2, h, (float)(mid * scale + oy)) < -band) lo = mid + 1;
            else hi = mid;
        }
        ya = lo;
        hi = G::FD;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (!(fmaf(-amp2, h, (float)(mid * scale + oy)) > band)) lo = mid + 1;
            else hi = mid;
        }
        yb = lo;
    }
    // the warp's row words of the rows decided solid: every valid column is
    // solid below the warp's lowest ya and none from its highest, so only the
    // rows between need a ballot.  Lane l keeps rows l, l + 32 and l + 64.
    {
        const unsigned vmask = __ballot_sync(FULL, valid);
        const int ymin = __reduce_min_sync(FULL, valid ? ya : G::FD);
        const int ymax = __reduce_max_sync(FULL, valid ? ya : 0);
        uint32_t w0 = 0, w1 = 0, w2 = 0;
        for (int y = ymin; y < ymax; y++) {
            const unsigned sb = __ballot_sync(FULL, y < ya);
            if ((y & 31) == lane) {
                w0 = y < 32 ? sb : w0;
                w1 = y >= 32 && y < 64 ? sb : w1;
                w2 = y >= 64 ? sb : w2;
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int y = lane + 32 * k;
            if (y < G::FD) words[warp][y] = y < ymin ? vmask : y >= ymax ? 0u : k == 0 ? w0 : k == 1 ? w1 : w2;
        }
    }
    // list the band rows of every column: an exclusive scan of the counts
    const int cnt = valid ? yb - ya : 0;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int off = incl - cnt;
    for (int w = 0; w < warp; w++) off += wsum[w];
    const int nl = wsum[0] + wsum[1] + wsum[2];
    for (int k = 0; k < cnt; k++) list[off + k] = (uint16_t)(x + G::FD * (ya + k));
    __syncthreads();
    // The listed points, a batch at a time, two fBm octaves a step.  After a
    // step, a point whose partial density fma(amp3, noise, base) exceeds the
    // bound on the octaves still to come (b.cave_rem) in magnitude keeps that
    // sign whatever they add, so it is decided; the others carry their partial
    // sum (the exact float the full loop holds there) to the next step through
    // a compacted batch list, and the last step decides by the full density.
    const int steps = dp.octaves3 > 0 ? (dp.octaves3 + 1) / 2 : 1;
    for (int b0 = 0; b0 < nl; b0 += kCaveBatch) {
        const int nb = min(kCaveBatch, nl - b0);
        for (int st = 0; st < steps; st++) {
            const int src = st & 1, dst = src ^ 1;
            const int n_in = st == 0 ? nb : bcount[src];
            __syncthreads();  // every thread has read n_in
            if (threadIdx.x == 0) bcount[dst] = 0;
            __syncthreads();
            const bool last = st + 1 == steps;
            const float rem = b.cave_rem[st + 1];
            for (int k = threadIdx.x; k < n_in; k += blockDim.x) {
                const int i = st == 0 ? list[b0 + k] : bidx[src][k];
                const int y = i / G::FD, px = i - G::FD * y;
                const float wy = (float)(y * scale + oy);
                const float base = fmaf(-amp2, hs[px], wy);
                const float noise = nz.fbm3_step(st, dp.octaves3, dp.freq3, dp.lacunarity3, dp.gain3,
                                                 (float)(px * scale + ox), wy, wz, st == 0 ? 0.f : bnoise[src][k]);
                const float v = fmaf(dp.amp3, noise, base);
                if (last || !(fabsf(v) <= rem)) {
                    if (v < 0.f) atomicOr(&words[px >> 5][y], 1u << (px & 31));
                } else {
                    const int slot = atomicAdd(&bcount[dst], 1);
                    bidx[dst][slot] = (uint16_t)i;
                    bnoise[dst][slot] = noise;
                }
            }
            __syncthreads();
            if (bcount[dst] == 0) break;
        }
    }
    __syncthreads();
    const uint4 V = low_bits(G::FD);
    uint4* P = plane_ptr<VPC>(b, c, 0) + G::FD * z;
    uint4* A = plane_ptr<VPC>(b, c, 1) + G::FD * z;
    uint4* X = plane_ptr<VPC>(b, c, 2) + G::FD * z;
    for (int y = threadIdx.x; y < G::FD; y += blockDim.x) {
        const uint4 p = make_uint4(words[0][y], words[1][y], words[2][y], 0u);
        P[y] = p;
        A[y] = and4(not4(p), V);
        X[y] = make_uint4(0u, 0u, 0u, 0u);
    }
    // byte materials, where the batch keeps them: the default material where
    // the point is solid, AIR elsewhere
    if (b.need_mats && valid) {
        uint8_t* mats = b.mats + (size_t)c * G::F + x + G::FD * G::FD * z;
        const uint32_t* wc = &words[x >> 5][0];
        const uint32_t bit = 1u << (x & 31);
        for (int y = 0; y < G::FD; y++) mats[G::FD * y] = (uint8_t)((wc[y] & bit) ? dm : MATERIAL_AIR);
    }
}

// Field of a chunk that takes the learned surrogate's densities (density
// < 0 is solid, as DensityFunc's sign is read by GenerateDefaultField).
template <int VPC>
__global__ void __launch_bounds__(128) k_field_sdens(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ uint32_t words[3][G::FD];
    const int c = blockIdx.y, z = blockIdx.x;
    const int slot = b.sslot[c];
    if (slot < 0) return;
    for (int i = threadIdx.x; i < 3 * G::FD; i += blockDim.x) (&words[0][0])[i] = 0u;
    __syncthreads();
    const float* dens = b.sdens + (size_t)slot * G::F + (size_t)G::FD * G::FD * z;
    const int dm = b.default_material;
    const bool write_mats = b.need_mats != 0;
    uint8_t* mats = b.mats + (size_t)c * G::F + G::FD * G::FD * z;
    for (int i = threadIdx.x; i < G::FD * G::FD; i += blockDim.x) {
        const int y = i / G::FD, x = i - G::FD * y;
        const int m = dens[i] < 0.f ? dm : MATERIAL_AIR;
        if (write_mats) mats[i] = (uint8_t)m;
        if (m != MATERIAL_AIR) atomicOr(&words[x >> 5][y], 1u << (x & 31));
    }
    __syncthreads();
    const uint4 V = low_bits(G::FD);
    uint4* P = plane_ptr<VPC>(b, c, 0) + G::FD * z;
    uint4* A = plane_ptr<VPC>(b, c, 1) + G::FD * z;
    uint4* X = plane_ptr<VPC>(b, c, 2) + G::FD * z;
    for (int y = threadIdx.x; y < G::FD; y += blockDim.x) {
        const uint4 p = make_uint4(words[0][y], words[1][y], words[2][y], 0u);
        P[y] = p;
        A[y] = and4(not4(p), V);
        X[y] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// 8 x 8 x 8 probes per chunk at field points (FD - 1) * (2i + 1) / 16, with
// the plain density there
template <int VPC>
__global__ void __launch_bounds__(kProbes) k_probe(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ __align__(16) float sg[64];
    stage_gradients(sg, b.grad);
    __syncthreads();
    const int c = blockIdx.x, p = threadIdx.x;
    const ChunkDesc& d = b.desc[c];
    const int ix = (G::FD - 1) * (2 * (p & 7) + 1) / 16, iy = (G::FD - 1) * (2 * ((p >> 3) & 7) + 1) / 16,
              iz = (G::FD - 1) * (2 * (p >> 6) + 1) / 16;
    const float wx = (float)(d.off[0] + d.scale * ix), wy = (float)(d.off[1] + d.scale * iy),
                wz = (float)(d.off[2] + d.scale * iz);
    const Noise nz{b.perm_t3, sg};
    b.probe_pts[(size_t)c * kProbes + p] = make_float4(wx, wy, wz, 0.f);
    b.probe_plain[(size_t)c * kProbes + p] = nz.density(b.density, wx, wy, wz);
}

__global__ void __launch_bounds__(kProbes) k_gate(BatchPtrs b) {
    __shared__ int bad;
    const int c = blockIdx.x, p = threadIdx.x;
    if (p == 0) bad = 0;
    __syncthreads();
    const size_t i = (size_t)c * kProbes + p;
    // the gate is in voxels of the chunk: scale density units per voxel
    if (!(fabsf(b.probe_s[i] - b.probe_plain[i]) <= b.gate * (float)b.desc[c].scale)) bad = 1;
    __syncthreads();
    if (p == 0) b.gate_ok[c] = bad ? 0 : 1;
}

// A persistent grid over the batch's (chunk, z slice) pairs, pair w to CTA
// w % gridDim.x.  On a large batch few slices have work (the chunks an
// operation touches, inside their operation boxes), so a CTA first tests a
// block of its pairs with one thread each and lists those with work, then
// takes the listed slices one at a time: 96 threads along x (three warps,
// one per plane word) times kCsgRows rows of y taken together.  One CTA per
// pair instead launched n * 66 CTAs, nearly all of them empty on a clipmap
// batch.
constexpr int kCsgRows = 8;
constexpr int kCsgThreads = 96 * kCsgRows;

template <int VPC>
__global__ void __launch_bounds__(kCsgThreads) k_csg(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int active[kCsgThreads];
    __shared__ int nact;
    const int tid = threadIdx.x + 96 * threadIdx.y;
    const int items = b.n * G::FD;
    const int mine = (items - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;  // this CTA's pairs
    for (int base = 0; base < mine; base += kCsgThreads) {
        if (tid == 0) nact = 0;
        __syncthreads();
        const int k = base + tid;
        const int w = (int)blockIdx.x + k * (int)gridDim.x;
        if (k < mine) {
            const int c = w / G::FD, z = w - G::FD * c;
            const ChunkDesc& dd = b.desc[c];
            if (dd.op_count > 0 && z >= dd.csg_lo[2] && z <= dd.csg_hi[2]) active[atomicAdd(&nact, 1)] = w;
        }
        __syncthreads();
        const int na = nact;
        for (int a = 0; a < na; a++) {
            const int c = active[a] / G::FD, z = active[a] - G::FD * (active[a] / G::FD);
            const ChunkDesc d = b.desc[c];  // a copy: the byte stores below may alias the descriptor
            const int nops = d.op_count;
            const int x = threadIdx.x;
            const bool inx = x < G::FD && x >= d.csg_lo[0] && x <= d.csg_hi[0];
            const Brush* ops = b.brushes + d.op_begin;
            uint8_t* mats = b.mats + (size_t)c * G::F + G::FD * G::FD * z;
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            uint32_t* A = reinterpret_cast<uint32_t*>(plane_ptr<VPC>(b, c, 1) + G::FD * z);
            uint32_t* X = reinterpret_cast<uint32_t*>(plane_ptr<VPC>(b, c, 2) + G::FD * z);
            const float wx = (float)(d.off[0] + d.scale * x);
            const float wz = (float)(d.off[2] + d.scale * z);
            for (int y = d.csg_lo[1] + (int)threadIdx.y; y <= d.csg_hi[1]; y += kCsgRows) {  // uniform per warp
                bool air = false, changed = false;
                if (x < G::FD) {
                    // a fresh field's materials are the default or AIR, given by its
                    // plain-solid bits; a cached field's are in the byte array
                    const int m = b.need_mats ? mats[x + G::FD * y]
                                              : (bit4(plane_ptr<VPC>(b, c, 0)[y + G::FD * z], x) ? b.default_material
                                                                                                : MATERIAL_AIR);
                    int nm = m;
                    if (inx) {
                        const float wy = (float)(d.off[1] + d.scale * y);
                        for (int i = 0; i < nops; i++) {
                            const Brush& br = ops[i];
                            if (brush_density(br, wx, wy, wz) <= 0.f) nm = br.type == 0 ? br.material : MATERIAL_AIR;
                        }
                        // inside the box the byte array holds the final material
                        if (nm != m || !b.need_mats) mats[x + G::FD * y] = (uint8_t)nm;
                    }
                    air = nm == MATERIAL_AIR;
                    changed = nm != m;
                }
                const unsigned aw = __ballot_sync(FULL, air), cw = __ballot_sync(FULL, changed);
                if (lane == 0) {
                    A[4 * y + warp] = aw;
                    X[4 * y + warp] = cw;
                }
            }
        }
        __syncthreads();  // every thread is done with the list before the next block resets it
    }
}

// ---------------------------------------------------------------------------
// Cached-field CSG (compute_csg.cpp:140-175): the field's existing edges that
// no changed corner touches are kept, in order, ahead of the created edges.
// One CTA, chunk 0 of a one-chunk batch.
// ---------------------------------------------------------------------------

template <int VPC>
__global__ void __launch_bounds__(1024) k_prune_edges(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[1024 / 32 + 1];
    const uint4* X = plane_ptr<VPC>(b, 0, 2);
    const int n = b.prev_count;
    int base = 0;
    for (int r = 0; r < n; r += 1024) {
        const int i = r + threadIdx.x;
        int keep = 0;
        int key = 0;
        if (i < n) {
            key = b.prev_keys[i];
            const int a = key & 3, h = key >> 2;
            const int x = h & G::MASK, y = (h >> G::SHIFT) & G::MASK, z = (h >> (2 * G::SHIFT)) & G::MASK;
            const int row = y + G::FD * z;
            bool touched = bit4(X[row], x);
            if (a == 0 && x + 1 < G::FD) touched = touched || bit4(X[row], x + 1);
            if (a == 1 && y + 1 < G::FD) touched = touched || bit4(X[row + 1], x);
            if (a == 2 && z + 1 < G::FD) touched = touched || bit4(X[row + G::FD], x);
            keep = touched ? 0 : 1;
        }
        int total;
        const int ex = block_exclusive<1024>(keep, total, sm);
        if (keep && base + ex < b.ecap) {
            b.edge_keys[base + ex] = key;
            b.edge_info[base + ex] = b.prev_info[i];
            b.edge_chunk[base + ex] = 0;
        }
        base += total;
    }
    if (threadIdx.x == 0) b.cs[0].kept_edges = base;
}

// ---------------------------------------------------------------------------
// stage 3-5: field edges, one thread per field row.  For point q, axis a:
//   plain-kept = q in the hermite grid, the plain field changes sign along a
//                and no CSG-changed corner touches the edge;
//   created    = the edge is touched (FindUpdatedEdges: a changed end point,
//                the far end only when it is a real field point) and the
//                final materials change sign along it (FilterValidEdges,
//                reading the linear successor with the PARANOID guard).
// ---------------------------------------------------------------------------

struct RowEdges {
    uint4 kept[3];
    uint4 created[3];
};

template <int VPC>
__device__ __forceinline__ RowEdges row_edges(const BatchPtrs& b, int c, int row) {
    using G = Geo<VPC>;
    constexpr int R = G::FD * G::FD;
    const int y = row % G::FD, z = row / G::FD;
    const uint4* P = plane_ptr<VPC>(b, c, 0);
    const uint4* A = plane_ptr<VPC>(b, c, 1);
    const uint4* X = plane_ptr<VPC>(b, c, 2);
    const uint4 V = low_bits(G::FD);
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    const uint4 a0 = A[row], x0 = X[row];
    const bool has_y = row + 1 < R, has_z = row + G::FD < R;
    const uint4 a_next = has_y ? A[row + 1] : V;
    const uint4 a_up = has_z ? A[row + G::FD] : V;
    const uint4 x_y = (y + 1 < G::FD) ? X[row + 1] : zero;
    const uint4 x_z = (z + 1 < G::FD) ? X[row + G::FD] : zero;
    // final-air neighbours: x + 1 (linear successor at x = FD-1), y + 1, z + 1
    uint4 ax = shr1(a0);
    if (bit4(a_next, 0)) ax = or4(ax, xor4(low_bits(G::FD), low_bits(G::FD - 1)));
    const uint4 t0 = or4(x0, shr1(x0)), t1 = or4(x0, x_y), t2 = or4(x0, x_z);
    RowEdges e;
    e.created[0] = and4(and4(t0, xor4(a0, ax)), V);
    e.created[1] = and4(and4(t1, xor4(a0, a_next)), V);
    e.created[2] = and4(and4(t2, xor4(a0, a_up)), V);
    if (b.plain_class && y < G::HD && z < G::HD) {
        const uint4 H = low_bits(G::HD);
        const uint4 p0 = P[row];
        e.kept[0] = and4(and4(H, xor4(p0, shr1(p0))), not4(t0));
        e.kept[1] = and4(and4(H, xor4(p0, P[row + 1])), not4(t1));
        e.kept[2] = and4(and4(H, xor4(p0, P[row + G::FD])), not4(t2));
    } else {
        e.kept[0] = e.kept[1] = e.kept[2] = zero;
    }
    return e;
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_edge_count(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[kThreads / 32 + 1];
    const int c = blockIdx.y, tile = blockIdx.x;
    const int row = tile * kThreads + threadIdx.x;
    int plain = 0, created = 0;
    if (row < G::FD * G::FD) {
        const RowEdges e = row_edges<VPC>(b, c, row);
        plain = (popc4(e.kept[0]) + popc4(e.kept[2])) | (popc4(e.kept[1]) << 16);
        created = popc4(e.created[0]) + popc4(e.created[1]) + popc4(e.created[2]);
    }
    const int tp = block_sum<kThreads>(plain, sm);
    const int tc = block_sum<kThreads>(created, sm);
    if (threadIdx.x == 0) b.edge_tiles[(size_t)c * G::NBE + tile] = make_int4(tp & 0xffff, tp >> 16, tc, 0);
}

// Exclusive scan over one warp; the smallest prime >= n (FindNextPrime,
// primes.cpp:32-58: candidates 6k +- 1, trial division), 32 candidates at a time.
__device__ __forceinline__ int warp_find_next_prime(int n) {
    if (n <= 2) return 2;
    if (n == 3) return 3;
    if (n <= 5) return 5;
    const int lane = threadIdx.x & 31;
    const int k = n / 6;
    const int o = (n - 6 * k) < 2 ? 1 : 5;
    const int x0 = 6 * k + o;
    for (int base = 0;; base += 32) {
        const int j = base + lane;
        const int cand = x0 + 6 * (j >> 1) + ((j & 1) ? (o == 1 ? 4 : 2) : 0);
        const unsigned m = __ballot_sync(FULL, is_prime_d(cand));
        if (m) return __shfl_sync(FULL, cand, __ffs(m) - 1);
    }
}

// Slots reserved for a chunk's cuckoo table of k keys: its prime
// (nextprime(max(2048, 2k)), compute_cuckoo.cpp:53) is below that bound plus
// 512 (prime gaps below 2^31 are under 300), then the 101-entry stash.
__device__ __forceinline__ int table_slot_bound(int k) {
    return k > 0 ? max((int)CUCKOO_MIN_TABLE_SIZE, 2 * k) + 512 + CUCKOO_STASH_SIZE : 0;
}

// The two cuckoo primes of every chunk, one warp per chunk.
__global__ void __launch_bounds__(256) k_primes(BatchPtrs b) {
    if (b.bs->overflow) return;
    const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (c >= b.n) return;
    ChunkState& st = b.cs[c];
    const int e = st.num_edges, v = st.nodes;
    const int pe = e > 0 ? warp_find_next_prime(max((int)CUCKOO_MIN_TABLE_SIZE, 2 * e)) : 0;
    const int pv = v > 0 ? warp_find_next_prime(max((int)CUCKOO_MIN_TABLE_SIZE, 2 * v)) : 0;
    if ((threadIdx.x & 31) == 0) {
        st.edge_prime = (uint32_t)pe;
        st.node_prime = (uint32_t)pv;
        st.edge_magic = pe ? 0xffffffffu / (uint32_t)pe : 0u;
        st.node_magic = pv ? 0xffffffffu / (uint32_t)pv : 0u;
    }
}

// The edge plan in two launches: per-chunk tile offsets (many CTAs), then the
// batch's per-chunk edge offsets and edge-table plan (one CTA).
// Each chunk's edge tiles: exclusive offsets of the three edge classes within
// the chunk and the chunk's counts.  One warp per chunk, eight chunks a CTA.
template <int VPC>
__global__ void __launch_bounds__(256) k_edge_tiles(BatchPtrs b) {
    using G = Geo<VPC>;
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (c >= b.n) return;  // the warp's own chunk: the exit is warp-uniform
    int4* t = b.edge_tiles + (size_t)c * G::NBE;
    int cx = 0, cy = 0, cc = 0;
    for (int base = 0; base < G::NBE; base += 32) {
        const int i = base + lane;
        const int4 v = i < G::NBE ? t[i] : make_int4(0, 0, 0, 0);
        const int ix = warp_inclusive(v.x), iy = warp_inclusive(v.y), ic = warp_inclusive(v.z);
        if (i < G::NBE) t[i] = make_int4(cx + ix - v.x, cy + iy - v.y, cc + ic - v.z, 0);
        cx += __shfl_sync(FULL, ix, 31);
        cy += __shfl_sync(FULL, iy, 31);
        cc += __shfl_sync(FULL, ic, 31);
    }
    if (lane == 0) {
        // edges kept from a cached field precede the plain class
        const int cp = b.cs[c].kept_edges + cx + cy;
        b.cs[c].edges_xz = cx;
        b.cs[c].edges_y = cy;
        b.cs[c].plain_edges = cp;
        b.cs[c].created_edges = cc;
        b.cs[c].num_edges = cp + cc;
    }
}

// Exclusive scans of K values a thread over the CTA, side by side with one
// set of barriers; `sm` holds K * (NT / 32 + 1) ints.
template <int NT, int K>
__device__ __forceinline__ void block_exclusive_k(const int (&v)[K], int (&ex)[K], int (&total)[K], int* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = NT / 32;
    int inc[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        inc[k] = warp_inclusive(v[k]);
        if (lane == 31) sm[k * (W + 1) + warp] = inc[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int w = lane < W ? sm[k * (W + 1) + lane] : 0;
            const int wi = warp_inclusive(w);
            if (lane < W) sm[k * (W + 1) + lane] = wi - w;
            if (lane == W - 1) sm[k * (W + 1) + W] = wi;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
        ex[k] = inc[k] - v[k] + sm[k * (W + 1) + warp];
        total[k] = sm[k * (W + 1) + W];
    }
    __syncthreads();
}

// The batch's edge offsets: five exclusive scans over the chunks in one pass
// (edges, hash-table slots, and the work-list segments of plain x / z, plain
// y and created edges), then the totals and the capacity checks.
template <int VPC>
__global__ void __launch_bounds__(1024) k_edge_plan(BatchPtrs b) {
    __shared__ int sm[5 * (1024 / 32 + 1)];
    long long carry[5] = {0, 0, 0, 0, 0};
    for (int base = 0; base < b.n; base += 1024) {
        const int c = base + threadIdx.x;
        int v[5] = {0, 0, 0, 0, 0};
        if (c < b.n) {
            const ChunkState& cs = b.cs[c];
            v[0] = cs.num_edges;
            // table slots are reserved for the largest prime the chunk can
            // need; the prime itself is found later by k_primes
            v[1] = table_slot_bound(cs.num_edges);
            v[2] = cs.edges_xz;
            v[3] = cs.edges_y;
            v[4] = cs.created_edges;
        }
        int ex[5], tot[5];
        block_exclusive_k<1024, 5>(v, ex, tot, sm);
        if (c < b.n) {
            ChunkState& cs = b.cs[c];
            cs.edge_off = (int)(carry[0] + ex[0]);
            cs.edge_table_off = (int)(carry[1] + ex[1]);
            cs.wl_xz_off = (int)(carry[2] + ex[2]);
            cs.wl_y_off = (int)(carry[3] + ex[3]);
            cs.wl_c_off = (int)(carry[4] + ex[4]);
        }
#pragma unroll
        for (int k = 0; k < 5; k++) carry[k] += tot[k];
    }
    if (threadIdx.x == 0) {
        b.bs->total_xz = (int)carry[2];
        b.bs->total_y = (int)carry[3];
        b.bs->total_created = (int)carry[4];
        b.bs->total_edges = (int)carry[0];
        b.bs->total_edge_slots = carry[1];
        int ovf = 0;
        if (carry[0] > b.ecap) ovf |= OVF_EDGES;
        if (carry[1] > b.edge_slot_cap) ovf |= OVF_EDGE_SLOTS;
        b.bs->overflow |= ovf;
    }
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_edge_scatter(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[kThreads / 32 + 1];
    if (b.bs->overflow) return;
    const int c = blockIdx.y, tile = blockIdx.x;
    const int row = tile * kThreads + threadIdx.x;
    const bool valid = row < G::FD * G::FD;
    RowEdges e;
    int nxz = 0, ny = 0, nc = 0;
    if (valid) {
        e = row_edges<VPC>(b, c, row);
        nxz = popc4(e.kept[0]) + popc4(e.kept[2]);
        ny = popc4(e.kept[1]);
        nc = popc4(e.created[0]) + popc4(e.created[1]) + popc4(e.created[2]);
    }
    int tp, tc;
    const int exp = block_exclusive<kThreads>(nxz | (ny << 16), tp, sm);
    const int exc = block_exclusive<kThreads>(nc, tc, sm);
    if (!valid || (nxz | ny | nc) == 0) return;
    const ChunkState st = b.cs[c];
    const BatchState& bs = *b.bs;
    const int4 toff = b.edge_tiles[(size_t)c * G::NBE + tile];
    const int exz = exp & 0xffff, ey = exp >> 16;
    int pp = st.edge_off + st.kept_edges + toff.x + toff.y + exz + ey;
    int pc = st.edge_off + st.plain_edges + toff.z + exc;
    int wxz = st.wl_xz_off + toff.x + exz;
    int wy = bs.total_xz + st.wl_y_off + toff.y + ey;
    int wc = bs.total_xz + bs.total_y + st.wl_c_off + toff.z + exc;
    const int y = row % G::FD, z = row / G::FD;
    // emit in (x, axis) order, the reference's (hermite index, axis) order:
    // word by word (x = 32 w + bit), lowest set bit first
    static_assert(G::FD <= 96, "a field row spans at most three 32-bit words");
    auto word = [](const uint4& u, int w) { return w == 0 ? u.x : w == 1 ? u.y : u.z; };
#pragma unroll
    for (int w = 0; w < 3; w++) {
        const uint32_t k0 = word(e.kept[0], w), k1 = word(e.kept[1], w), k2 = word(e.kept[2], w);
        for (uint32_t any = k0 | k1 | k2; any; any &= any - 1) {
            const int bit = __ffs(any) - 1, x = 32 * w + bit;
            if ((k0 >> bit) & 1) {
                b.edge_keys[pp] = edge_key<VPC>(x, y, z, 0);
                b.edge_chunk[pp] = c;
                b.edge_work[wxz++] = pp++;
            }
            if ((k1 >> bit) & 1) {
                b.edge_keys[pp] = edge_key<VPC>(x, y, z, 1);
                b.edge_chunk[pp] = c;
                b.edge_work[wy++] = pp++;
            }
            if ((k2 >> bit) & 1) {
                b.edge_keys[pp] = edge_key<VPC>(x, y, z, 2);
                b.edge_chunk[pp] = c;
                b.edge_work[wxz++] = pp++;
            }
        }
    }
#pragma unroll
    for (int w = 0; w < 3; w++) {
        const uint32_t c0 = word(e.created[0], w), c1 = word(e.created[1], w), c2 = word(e.created[2], w);
        for (uint32_t any = c0 | c1 | c2; any; any &= any - 1) {
            const int bit = __ffs(any) - 1, x = 32 * w + bit;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (((a == 0 ? c0 : a == 1 ? c1 : c2) >> bit) & 1) {
                    b.edge_keys[pc] = edge_key<VPC>(x, y, z, a);
                    b.edge_chunk[pc] = c;
                    b.edge_work[wc++] = pc++;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// stage 6: hermite data per edge
// ---------------------------------------------------------------------------

// FindEdgeIntersectionInfo (density_field.cl:96-151).  A y edge keeps x and z
// fixed, so its height term is evaluated once; the other edges evaluate it
// per sample.  Each density evaluation has one call site in a loop, which
// keeps the kernel small enough for the instruction cache.
// `hm` is the chunk's height map (the field kernel's height term per column),
// or null: the height at an edge's end points is then read, not recomputed,
// with the same arguments and so the same value.
template <int VPC, int MODE, class N>
__device__ __forceinline__ float4 hermite_density(const BatchPtrs& b, const N& nz, const ChunkDesc& d, int key,
                                                  const float* hm) {
    using G = Geo<VPC>;
    const int axis = key & 3;
    const int hidx = key >> 2;
    const int lx = hidx & G::MASK, ly = (hidx >> G::SHIFT) & G::MASK, lz = (hidx >> (2 * G::SHIFT)) & G::MASK;
    const int s = d.scale;
    const int wx = s * lx + d.off[0], wy = s * ly + d.off[1], wz = s * lz + d.off[2];
    const float p0x = (float)wx, p0y = (float)wy, p0z = (float)wz;
    const float p1x = (float)(wx + (axis == 0 ? s : 0));
    const float p1y = (float)(wy + (axis == 1 ? s : 0));
    const float p1z = (float)(wz + (axis == 2 ? s : 0));
    const DensityParams& dp = b.density;
    const bool yedge = axis == 1;
    float t = 0.f;
    float hbest = 0.f;
    if (b.crossing_mode == 0) {
        // 17-sample search for min |d| (density_field.cl:122-136); first minimum wins
        float minv = FLT_MAX;
        float cur = 0.f;
        // the end points are field columns: (lx, lz) and (lx, lz) + the x or z step
        const int c0 = lx + G::FD * lz, c1 = c0 + (axis == 0 ? 1 : axis == 2 ? G::FD : 0);
        float hy = 0.f;
        if (yedge) hy = hm ? hm[c0] : height_m<MODE>(nz, dp, p0x, p0z);
        for (int i = 0; i <= 16; i++) {
            const float px = fmaf(p1x - p0x, cur, p0x);
            const float py = fmaf(p1y - p0y, cur, p0y);
            const float pz = fmaf(p1z - p0z, cur, p0z);
            // t = 0 and t = 1 (cur sums 16 exact 1/16 steps) land on the end points
            const float h = yedge ? hy
                            : (hm && (i == 0 || i == 16)) ? hm[i == 0 ? c0 : c1]
                                                          : height_m<MODE>(nz, dp, px, pz);
            const float dv = fabsf(dens_h<MODE>(nz, dp, h, px, py, pz));
            if (dv < minv) { t = cur; minv = dv; hbest = h; }
            cur += 0.0625f;
        }
    } else {
        float e0 = 0.f, e1 = 0.f;
        for (int j = 0; j < 2; j++) {
            const float qx = j ? p1x : p0x, qy = j ? p1y : p0y, qz = j ? p1z : p0z;
            const float v = dens_h<MODE>(nz, dp, height_m<MODE>(nz, dp, qx, qz), qx, qy, qz);
            e0 = j == 0 ? v : e0;
            e1 = j == 1 ? v : e1;
        }
        const float den = e0 - e1;
        t = den != 0.f ? e0 / den : 0.5f;
        t = fminf(fmaxf(t, 0.f), 1.f);
        hbest = height_m<MODE>(nz, dp, fmaf(p1x - p0x, t, p0x), fmaf(p1z - p0z, t, p0z));
    }
    const float px = fmaf(p1x - p0x, t, p0x);
    const float py = fmaf(p1y - p0y, t, p0y);
    const float pz = fmaf(p1z - p0z, t, p0z);
    const float h = 0.001f;
    // central differences: x+h, x-h, z+h, z-h need their own height term;
    // y+h and y-h share the one at (px, pz)
    float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;  // registers, not an indexed array
    for (int j = 0; j < 4; j++) {
        const float qx = j == 0 ? px + h : j == 1 ? px - h : px;
        const float qz = j == 2 ? pz + h : j == 3 ? pz - h : pz;
        const float v = dens_h<MODE>(nz, dp, height_m<MODE>(nz, dp, qx, qz), qx, py, qz);
        d0 = j == 0 ? v : d0;
        d1 = j == 1 ? v : d1;
        d2 = j == 2 ? v : d2;
        d3 = j == 3 ? v : d3;
    }
    float ny0 = 0.f, ny1 = 0.f;
    for (int j = 0; j < 2; j++) {
        const float v = dens_h<MODE>(nz, dp, hbest, px, j ? py - h : py + h, pz);
        ny0 = j == 0 ? v : ny0;
        ny1 = j == 1 ? v : ny1;
    }
    float nx = d0 - d1;
    float ny = ny0 - ny1;
    float nzv = d2 - d3;
    normalize3(nx, ny, nzv);
    return make_float4(nx, ny, nzv, t);
}

// CSG FindEdgeIntersectionInfo (apply_csg_operation.cl:443-477)
template <int VPC>
__device__ __forceinline__ float4 hermite_brush(const BatchPtrs& b, const ChunkDesc& d, int key) {
    using G = Geo<VPC>;
    const int axis = key & 3;
    const int hidx = key >> 2;
    const int lx = hidx & G::MASK, ly = (hidx >> G::SHIFT) & G::MASK, lz = (hidx >> (2 * G::SHIFT)) & G::MASK;
    const int s = d.scale;
    const int wx = s * lx + d.off[0], wy = s * ly + d.off[1], wz = s * lz + d.off[2];
    const float p0x = (float)wx, p0y = (float)wy, p0z = (float)wz;
    const float p1x = (float)(wx + (axis == 0 ? s : 0));
    const float p1y = (float)(wy + (axis == 1 ? s : 0));
    const float p1z = (float)(wz + (axis == 2 ? s : 0));
    const Brush* ops = b.brushes + d.op_begin;
    const int nops = d.op_count;
    // BrushZeroCrossing (apply_csg_operation.cl:86-110)
    float mind = FLT_MAX, t = 0.f;
    for (float tt = 0.f; tt <= 1.f; tt += (1.f / 16.f)) {
        const float px = fmaf(p1x - p0x, tt, p0x);
        const float py = fmaf(p1y - p0y, tt, p0y);
        const float pz = fmaf(p1z - p0z, tt, p0z);
        for (int i = 0; i < nops; i++) {
            const float dv = fabsf(brush_density(ops[i], px, py, pz));
            if (dv < mind) { t = tt; mind = dv; }
        }
    }
    const float px = fmaf(p1x - p0x, t, p0x);
    const float py = fmaf(p1y - p0y, t, p0y);
    const float pz = fmaf(p1z - p0z, t, p0z);
    // BrushNormal (apply_csg_operation.cl:144-175): the last containing op wins
    float nx = 0.f, ny = 0.f, nzv = 0.f;
    const float h = 0.001f;
    for (int i = 0; i < nops; i++) {
        const Brush& br = ops[i];
        if (brush_density(br, px, py, pz) > 0.f) continue;
        float gx = brush_density(br, px + h, py, pz) - brush_density(br, px - h, py, pz);
        float gy = brush_density(br, px, py + h, pz) - brush_density(br, px, py - h, pz);
        float gz = brush_density(br, px, py, pz + h) - brush_density(br, px, py, pz - h);
        normalize3(gx, gy, gz);
        const float flip = br.type == 0 ? 1.f : -1.f;
        nx = flip * gx;
        ny = flip * gy;
        nzv = flip * gz;
    }
    return make_float4(nx, ny, nzv, t);
}

// Hermite data of an edge of a surrogate chunk: crossing by linear
// interpolation of the end points' densities, normal from central
// differences of the density field (one-sided at the field's faces)
// interpolated to the crossing.
template <int VPC>
__device__ __forceinline__ float4 hermite_sdens(const BatchPtrs& b, int slot, int key) {
    using G = Geo<VPC>;
    const int axis = key & 3;
    const int hidx = key >> 2;
    const int lx = hidx & G::MASK, ly = (hidx >> G::SHIFT) & G::MASK, lz = (hidx >> (2 * G::SHIFT)) & G::MASK;
    const float* D = b.sdens + (size_t)slot * G::F;
    auto at = [&](int x, int y, int z) {
        x = min(max(x, 0), G::FD - 1);
        y = min(max(y, 0), G::FD - 1);
        z = min(max(z, 0), G::FD - 1);
        return D[x + G::FD * (y + G::FD * z)];
    };
    const int ox = axis == 0, oy = axis == 1, oz = axis == 2;
    const float d0 = at(lx, ly, lz), d1 = at(lx + ox, ly + oy, lz + oz);
    const float den = d0 - d1;
    float t = den != 0.f ? d0 / den : 0.5f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    float g[2][3];
#pragma unroll
    for (int e = 0; e < 2; e++) {
        const int x = lx + e * ox, y = ly + e * oy, z = lz + e * oz;
        g[e][0] = at(x + 1, y, z) - at(x - 1, y, z);
        g[e][1] = at(x, y + 1, z) - at(x, y - 1, z);
        g[e][2] = at(x, y, z + 1) - at(x, y, z - 1);
    }
    float nx = fmaf(g[1][0] - g[0][0], t, g[0][0]);
    float ny = fmaf(g[1][1] - g[0][1], t, g[0][1]);
    float nzv = fmaf(g[1][2] - g[0][2], t, g[0][2]);
    normalize3(nx, ny, nzv);
    return make_float4(nx, ny, nzv, t);
}

// The hermite work list, grid-stride: plain x/z edges, plain y edges,
// CSG-created edges, in segments, so that a warp's 32 edges take the same path.
template <int VPC, int MODE, class N>
__device__ __forceinline__ void hermite_list(const BatchPtrs& b, const N& nz) {
    const int nplain = b.bs->total_xz + b.bs->total_y;
    const int total = nplain + b.bs->total_created;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < total; w += gridDim.x * blockDim.x) {
        const int i = b.edge_work[w];
        const int c = b.edge_chunk[i];
        const ChunkDesc& d = b.desc[c];
        const int key = b.edge_keys[i];
        const int slot = b.s_on ? b.sslot[c] : -1;
        const float* hm = b.hmap ? b.hmap + (size_t)c * Geo<VPC>::FD * Geo<VPC>::FD : nullptr;
        b.edge_info[i] = w >= nplain ? hermite_brush<VPC>(b, d, key)
                         : slot >= 0 ? hermite_sdens<VPC>(b, slot, key)
                                     : hermite_density<VPC, MODE>(b, nz, d, key, hm);
    }
}

template <int VPC, int MODE>
__global__ void __launch_bounds__(kThreads) k_hermite(BatchPtrs b) {
    __shared__ __align__(16) float sg[64];
    stage_gradients(sg, b.grad);
    __syncthreads();
    if (b.bs->overflow) return;
    hermite_list<VPC, MODE>(b, Noise{b.perm_t3, sg});
}

// The same for large batches: one 1024-thread CTA per SM holds the two
// simplex lookup tables (kT3Bytes) in shared memory, so a table read is a
// shared load with a 32-bit address instead of a read-only global load with
// a 64-bit one (9% fewer instructions a 3D fBm).  Such a CTA takes an SM's
// registers and most of its shared memory, leaving the stages beside hermite
// in the batch DAG no room; on a large batch hermite's share of the step
// outweighs that, on a small one it does not.
template <int VPC, int MODE>
__global__ void __launch_bounds__(kHermiteSmemThreads, 1) k_hermite_smem(BatchPtrs b) {
    extern __shared__ __align__(16) uint8_t stab[];  // the lookup tables
    __shared__ __align__(16) float sg[64];
    if (b.bs->overflow) return;  // the same for every thread
    stage_gradients(sg, b.grad);
    const uint4* src = reinterpret_cast<const uint4*>(b.perm_t3);
    for (int i = threadIdx.x; i < kT3Bytes / 16; i += blockDim.x) reinterpret_cast<uint4*>(stab)[i] = __ldg(src + i);
    __syncthreads();
    hermite_list<VPC, MODE>(b, NoiseT<true>{stab, sg});
}

// ---------------------------------------------------------------------------
// stage 7-9: active voxels (FindActiveVoxels + CompactVoxels, octree.cl:142-223),
// one thread per voxel row (y, z) over the final-air plane.
// ---------------------------------------------------------------------------

struct VoxRow {
    uint4 s[4];    // solid rows (y,z), (y,z+1), (y+1,z), (y+1,z+1): corner bits i & 3
    uint4 active;
};

// corner i = CHILD_MIN_OFFSETS[i] = (i >> 2, (i >> 1) & 1, i & 1)
template <int VPC>
__device__ __forceinline__ VoxRow vox_row(const BatchPtrs& b, int c, int vrow) {
    using G = Geo<VPC>;
    const int y = vrow % VPC, z = vrow / VPC;
    const int r = y + G::FD * z;
    const uint4* A = plane_ptr<VPC>(b, c, 1);
    const uint4 V = low_bits(G::FD);
    VoxRow v;
    const uint4 a00 = A[r], a01 = A[r + G::FD], a10 = A[r + 1], a11 = A[r + G::FD + 1];
    v.s[0] = and4(not4(a00), V);
    v.s[1] = and4(not4(a01), V);
    v.s[2] = and4(not4(a10), V);
    v.s[3] = and4(not4(a11), V);
    uint4 all_s = make_uint4(~0u, ~0u, ~0u, ~0u), all_a = all_s;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        all_s = and4(all_s, and4(v.s[i], shr1(v.s[i])));
    }
    all_a = and4(and4(and4(a00, shr1(a00)), and4(a01, shr1(a01))), and4(and4(a10, shr1(a10)), and4(a11, shr1(a11))));
    v.active = and4(not4(or4(all_s, all_a)), low_bits(VPC));
    return v;
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_vox_count(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[kThreads / 32 + 1];
    const int c = blockIdx.y, tile = blockIdx.x;
    const int vrow = tile * kThreads + threadIdx.x;
    int cnt = 0;
    if (vrow < VPC * VPC) cnt = popc4(vox_row<VPC>(b, c, vrow).active);
    const int total = block_sum<kThreads>(cnt, sm);
    if (threadIdx.x == 0) b.vox_tiles[(size_t)c * G::NBV + tile] = total;
}

template <int VPC>
__global__ void __launch_bounds__(1024) k_vox_plan(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[1024 / 32 + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < b.n; c += 32) {
        // a chunk without field edges builds no octree (compute_octree.cpp:167-171)
        int v = warp_scan_array(b.vox_tiles + (size_t)c * G::NBV, G::NBV);
        if (b.cs[c].num_edges == 0) v = 0;
        if (lane == 0) b.cs[c].nodes = v;
    }
    __syncthreads();
    const long long total = cta_scan(
        b.n, [&](int c) { return b.cs[c].nodes; }, [&](int c, long long ex) { b.cs[c].node_off = (int)ex; }, nullptr, sm);
    const long long slots = cta_scan(
        b.n, [&](int c) { return table_slot_bound(b.cs[c].nodes); },
        [&](int c, long long ex) { b.cs[c].node_table_off = (int)ex; }, nullptr, sm);
    const long long tiles = cta_scan(
        b.n, [&](int c) { return (b.cs[c].nodes + kNodeTile - 1) / kNodeTile; },
        [&](int c, long long ex) { b.chunk_tile_off[c] = (int)ex; }, nullptr, sm);
    if (threadIdx.x == 0) {
        b.chunk_tile_off[b.n] = (int)tiles;
        b.bs->total_nodes = (int)total;
        b.bs->total_node_slots = slots;
        int ovf = 0;
        // with simplification the leaves go to leaf_out (vcap); the caller's
        // vertex array is checked against the simplified count
        if (total > b.vcap || (!b.simp_on && total > b.vertex_cap)) ovf |= OVF_NODES;
        if (slots > b.node_slot_cap) ovf |= OVF_NODE_SLOTS;
        if (tiles > b.node_tile_cap) ovf |= OVF_NODES;
        b.bs->overflow |= ovf;
    }
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_vox_scatter(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[kThreads / 32 + 1];
    if (b.bs->overflow) return;
    const int c = blockIdx.y, tile = blockIdx.x;
    const ChunkState& st = b.cs[c];
    if (st.nodes == 0) return;
    const int vrow = tile * kThreads + threadIdx.x;
    const bool valid = vrow < VPC * VPC;
    uint4 act = make_uint4(0u, 0u, 0u, 0u);
    if (valid) act = vox_row<VPC>(b, c, vrow).active;
    const int cnt = popc4(act);
    int total;
    const int ex = block_exclusive<kThreads>(cnt, total, sm);
    // the warp's active voxels, in row order then x order, are spread over
    // its lanes: voxel j of the warp goes to lane j % 32
    const int lane = threadIdx.x & 31;
    const int winc = warp_inclusive(cnt);
    const int wexcl = winc - cnt;
    const int wtotal = __shfl_sync(FULL, winc, 31);
    if (wtotal == 0) return;
    const int base = st.node_off + b.vox_tiles[(size_t)c * G::NBV + tile] + __shfl_sync(FULL, ex, 0);
    const uint4* A = plane_ptr<VPC>(b, c, 1);
    const uint8_t* mats = b.mats + (size_t)c * G::F;
    // a fresh field without CSG holds the default material or AIR only, so the
    // corner materials follow from the solid bits
    const bool fresh = b.derive_mats != 0;
    const bool has_ops = b.desc[c].op_count > 0;
    const int bx0 = b.desc[c].csg_lo[0], bx1 = b.desc[c].csg_hi[0], by0 = b.desc[c].csg_lo[1],
              by1 = b.desc[c].csg_hi[1], bz0 = b.desc[c].csg_lo[2], bz1 = b.desc[c].csg_hi[2];
    const int dm = b.default_material;
    for (int j0 = 0; j0 < wtotal; j0 += 32) {
        const int j = j0 + lane;
        // source lane: the last lane whose exclusive count is <= j
        int src = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int e = __shfl_sync(FULL, wexcl, (src + step) & 31);
            if (src + step < 32 && e <= j) src += step;
        }
        const int k = j - __shfl_sync(FULL, wexcl, src);
        const unsigned w0 = __shfl_sync(FULL, act.x, src), w1 = __shfl_sync(FULL, act.y, src);
        const int row = __shfl_sync(FULL, vrow, src);
        if (j >= wtotal) continue;
        // x of the k-th set bit of the source row
        unsigned w = w0;
        int kk = k, off = 0;
        if (kk >= __popc(w0)) { kk -= __popc(w0); w = w1; off = 32; }
        for (int i = 0; i < kk; i++) w &= w - 1;
        const int x = off + __ffs(w) - 1;
        const int y = row % VPC, z = row / VPC;
        const int r = y + G::FD * z;
        int corners = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int dx = i >> 2, dy = (i >> 1) & 1, dz = i & 1;
            corners |= (bit4(A[r + dy + G::FD * dz], x + dx) ? 0 : 1) << i;
        }
        int edges = 0;
#pragma unroll
        for (int i = 0; i < 12; i++) {
            const int s0 = (corners >> edge_c0(i)) & 1, s1 = (corners >> edge_c1(i)) & 1;
            edges |= (s0 != s1 ? 1 : 0) << i;
        }
        // a fresh field holds byte materials only inside its CSG box; a voxel
        // with every corner outside it has the default material at its solid
        // corners and AIR at the others, whose dominant material depends on
        // the solid count alone
        const bool outside = !has_ops || x + 1 < bx0 || x > bx1 || y + 1 < by0 || y > by1 || z + 1 < bz0 || z > bz1;
        int dom;
        if (fresh && outside) {
            dom = b.dom_by_solid[__popc(corners)];
        } else {
            int m[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int dx = i >> 2, dy = (i >> 1) & 1, dz = i & 1;
                const int cx = x + dx, cy = y + dy, cz = z + dz;
                const bool in_box =
                    has_ops && cx >= bx0 && cx <= bx1 && cy >= by0 && cy <= by1 && cz >= bz0 && cz <= bz1;
                m[i] = (fresh && !in_box) ? (((corners >> i) & 1) ? dm : MATERIAL_AIR)
                                          : mats[cx + G::FD * cy + G::FD * G::FD * cz];
            }
            dom = dominant_material(m);
        }
        const int pos = base + j;
        b.node_codes[pos] = code_for_position<VPC>(x, y, z);
        b.node_info[pos] = (edges << 16) | (dom << 8) | corners;
        b.node_chunk[pos] = c;
    }
}

// ---------------------------------------------------------------------------
// stage 10-13: cuckoo tables, leaves
// ---------------------------------------------------------------------------

__global__ void k_hash_fill(BatchPtrs b) {
    if (b.bs->overflow) return;
    const long long ne = b.bs->total_edge_slots, nn = b.bs->total_node_slots;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < ne + nn; i += stride) {
        if (i < ne) b.edge_slots[i] = CUCKOO_EMPTY;
        else b.node_slots[i - ne] = CUCKOO_EMPTY;
    }
}

__global__ void __launch_bounds__(kThreads) k_edge_insert(BatchPtrs b) {
    if (b.bs->overflow) return;
    const int total = b.bs->total_edges;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int c = b.edge_chunk[i];
        ChunkState* st = b.cs + c;
        const uint32_t prime = st->edge_prime;
        unsigned long long* table = b.edge_slots + st->edge_table_off;
        uint32_t p[10];
#pragma unroll
        for (int k = 0; k < 10; k++) p[k] = b.desc[c].edge_params[k];
        const int r = cuckoo_insert(table, table + prime, prime, st->edge_magic, p, (uint32_t)b.edge_keys[i],
                                    (uint32_t)(i - st->edge_off));
        if (r == 1) st->edge_stash_used = 1;
        if (r < 0) st->edge_insert_failed = 1;
    }
}

__global__ void __launch_bounds__(kThreads) k_node_insert(BatchPtrs b) {
    if (b.bs->overflow) return;
    const int total = b.bs->total_nodes;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int c = b.node_chunk[i];
        ChunkState* st = b.cs + c;
        const uint32_t prime = st->node_prime;
        unsigned long long* table = b.node_slots + st->node_table_off;
        uint32_t p[10];
#pragma unroll
        for (int k = 0; k < 10; k++) p[k] = b.desc[c].node_params[k];
        const int r = cuckoo_insert(table, table + prime, prime, st->node_magic, p, b.node_codes[i],
                                    (uint32_t)(i - st->node_off));
        if (r == 1) st->node_stash_used = 1;
        if (r < 0) st->node_insert_failed = 1;
    }
}

// Device-side repair of a chunk's cuckoo table after a failed insert (a key
// whose eviction chain ran out and whose stash slot was taken).  The host
// would redraw that chunk's parameters and rerun the whole batch; instead one
// CTA draws new parameters from the old ones, clears the table and inserts
// the chunk's keys again, up to kRepairAttempts times, within the batch.  The
// new parameters go to the chunk's descriptor, where the lookups read them.
// A chunk still failing after that keeps its flag, and the host reruns.
constexpr int kRepairAttempts = 8;
constexpr int kRepairThreads = 256;

// a parameter word from the previous one and a salt, in the host's draw
// range [2^15, 2^30] (a 32-bit finaliser of the two)
__device__ __forceinline__ uint32_t repair_param(uint32_t prev, uint32_t salt) {
    uint32_t x = prev ^ (salt * 0x9E3779B9u);
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return (1u << 15) + x % ((1u << 30) - (1u << 15) + 1u);
}

template <bool NODES>
__global__ void __launch_bounds__(kRepairThreads) k_hash_repair(BatchPtrs b) {
    __shared__ int list[kRepairThreads];
    __shared__ int nl, failed, stashed;
    if (b.bs->overflow) return;  // the same for every thread
    if (threadIdx.x == 0) nl = 0;
    __syncthreads();
    const int c = blockIdx.x * kRepairThreads + threadIdx.x;
    if (c < b.n && (NODES ? b.cs[c].node_insert_failed : b.cs[c].edge_insert_failed)) list[atomicAdd(&nl, 1)] = c;
    __syncthreads();
    for (int a = 0; a < nl; a++) {
        const int ch = list[a];
        ChunkState* st = b.cs + ch;
        // the descriptors are this batch's device copy: writable
        uint32_t* params = const_cast<uint32_t*>(NODES ? b.desc[ch].node_params : b.desc[ch].edge_params);
        const uint32_t prime = NODES ? st->node_prime : st->edge_prime;
        const uint32_t magic = NODES ? st->node_magic : st->edge_magic;
        unsigned long long* table = NODES ? b.node_slots + st->node_table_off : b.edge_slots + st->edge_table_off;
        const int first = NODES ? st->node_off : st->edge_off;
        const int count = NODES ? st->nodes : st->num_edges;
        for (int attempt = 0; attempt < kRepairAttempts; attempt++) {
            uint32_t p[10];
#pragma unroll
            for (int k = 0; k < 10; k++)  // an injected fault makes these degenerate too (a = 0)
                p[k] = b.hash_fault ? ((k & 1) ? 1u << 15 : 0u)
                                    : repair_param(params[k], (uint32_t)(ch * 10 + k) * 31u + (uint32_t)attempt);
            __syncthreads();  // every thread has read the previous parameters
            if (threadIdx.x < 10) params[threadIdx.x] = p[threadIdx.x];
            if (threadIdx.x == 0) {
                failed = 0;
                stashed = 0;
            }
            for (uint32_t i = threadIdx.x; i < prime + CUCKOO_STASH_SIZE; i += kRepairThreads) table[i] = CUCKOO_EMPTY;
            __syncthreads();
            for (int i = threadIdx.x; i < count; i += kRepairThreads) {
                const uint32_t key = NODES ? b.node_codes[first + i] : (uint32_t)b.edge_keys[first + i];
                const int r = cuckoo_insert(table, table + prime, prime, magic, p, key, (uint32_t)i);
                if (r == 1) stashed = 1;
                if (r < 0) failed = 1;
            }
            __syncthreads();
            if (!failed) break;
        }
        if (threadIdx.x == 0) {
            if (NODES) {
                st->node_stash_used = stashed;
                st->node_insert_failed = failed;
            } else {
                st->edge_stash_used = stashed;
                st->edge_insert_failed = failed;
            }
        }
        __syncthreads();  // the flags are read before the next chunk resets them
    }
}

// Test hook over an arbitrary key list: the same cuckoo_insert and
// HashView::find the meshing stages run (one table, value = key index).
__global__ void k_debug_cuckoo_fill(unsigned long long* table, int64_t slots) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += (int64_t)gridDim.x * blockDim.x)
        table[i] = CUCKOO_EMPTY;
}

__global__ void k_debug_cuckoo_insert(const uint32_t* keys, int n, unsigned long long* table, uint32_t prime,
                                      uint32_t magic, CuckooParams cp, int* status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = cuckoo_insert(table, table + prime, prime, magic, cp.p, keys[i], (uint32_t)i);
        if (r == 1) atomicOr(&status[0], 1);
        if (r < 0) atomicOr(&status[1], 1);
    }
}

__global__ void k_debug_cuckoo_find(const uint32_t* keys, int n, const unsigned long long* table, uint32_t prime,
                                    uint32_t magic, CuckooParams cp, const int* status, int reference_find,
                                    uint32_t* values) {
    HashView hv;
    hv.table = table;
    hv.stash = table + prime;
    hv.prime = prime;
    hv.magic = magic;
    hv.stash_used = status[0];
#pragma unroll
    for (int k = 0; k < 10; k++) hv.p[k] = cp.p[k];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        if (!reference_find) {
            values[i] = hv.find(key);
            continue;
        }
        // Cuckoo_Find as written: the stash probe reads data[h] (cuckoo.cl:93-101)
        uint32_t v = ~0u;
        for (int f = 0; f < CUCKOO_STASH_HASH_INDEX && v == ~0u; f++) {
            const unsigned long long e = table[cuckoo_hash(key, cp.p[2 * f], cp.p[2 * f + 1], prime, magic)];
            if ((uint32_t)e == key) v = (uint32_t)(e >> 32);
        }
        if (v == ~0u && hv.stash_used) {
            const unsigned long long e = table[stash_hash(key, cp.p[8], cp.p[9])];
            if ((uint32_t)e == key) v = (uint32_t)(e >> 32);
        }
        values[i] = v;
    }
}

// ---------------------------------------------------------------------------
// The FP32 leaf solve against an FP64 solve of the same crossings: the
// leaves' inputs gathered as k_leaf gathers them, qef_add_point
// (qef.cl:170-191) accumulated in double, and qef_solve (qef.cl:239-256) with
// its ten Jacobi sweeps, 0.1 truncation and mass-point bias in double.  The
// FP32 solve is the same qef_solve k_leaf runs on the same inputs.  Reports
// the distance in voxels of the leaf's chunk: max (as the bits of a
// non-negative double), sum, count, and the count above 1e-3 voxel.  A
// measurement pass, not a stage.
// ---------------------------------------------------------------------------

__device__ void qef_solve_f64(const double ata[6], const double atb[3], const double mpsum[4], double out[3]) {
    const double w = fmax(mpsum[3], 1.0);
    const double mp[3] = {mpsum[0] / w, mpsum[1] / w, mpsum[2] / w};
    const double amp[3] = {atb[0] - (ata[0] * mp[0] + ata[1] * mp[1] + ata[2] * mp[2]),
                           atb[1] - (ata[1] * mp[0] + ata[3] * mp[1] + ata[4] * mp[2]),
                           atb[2] - (ata[2] * mp[0] + ata[4] * mp[1] + ata[5] * mp[2])};
    double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double vt[3][3] = {{ata[0], ata[1], ata[2]}, {0, ata[3], ata[4]}, {0, 0, ata[5]}};
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    for (int it = 0; it < 10; it++)
        for (int r = 0; r < 3; r++) {
            const int a = pa[r], bq = pb[r];
            if (vt[a][bq] == 0.0) continue;
            const double tau = (vt[bq][bq] - vt[a][a]) / (2.0 * vt[a][bq]);
            const double stt = sqrt(1.0 + tau * tau);
            const double tn = 1.0 / (tau >= 0.0 ? tau + stt : tau - stt);
            const double c = 1.0 / sqrt(1.0 + tn * tn), sn = tn * c;
            const double cc = c * c, ss = sn * sn, mx = 2.0 * c * sn * vt[a][bq];
            const double u = vt[a][a], v = vt[bq][bq];
            vt[a][a] = cc * u - mx + ss * v;
            vt[bq][bq] = ss * u + mx + cc * v;
            const double x = vt[0][3 - bq], y = vt[1 - a][2];
            vt[0][3 - bq] = c * x - sn * y;
            vt[1 - a][2] = sn * x + c * y;
            vt[a][bq] = 0.0;
            for (int k = 0; k < 3; k++) {
                const double pv = V[k][a], qv = V[k][bq];
                V[k][a] = c * pv - sn * qv;
                V[k][bq] = sn * pv + c * qv;
            }
        }
    double d[3];
    for (int k = 0; k < 3; k++) {
        const double x = vt[k][k];
        d[k] = (fabs(x) < 0.1 || fabs(1.0 / x) < 0.1) ? 0.0 : 1.0 / x;
    }
    for (int r = 0; r < 3; r++) {
        double x = 0.0;
        for (int c = 0; c < 3; c++) x += (V[r][0] * d[0] * V[c][0] + V[r][1] * d[1] * V[c][1] + V[r][2] * d[2] * V[c][2]) * amp[c];
        out[r] = x + mp[r];
    }
}

template <int VPC>
__global__ void __launch_bounds__(256) k_leaf_qef_check(BatchPtrs b, unsigned long long* stats) {
    if (b.bs->overflow) return;
    const int total = b.bs->total_nodes;
    double local_max = 0.0, local_sum = 0.0;
    unsigned long long local_n = 0, local_far = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int c = b.node_chunk[i];
        const ChunkState& st = b.cs[c];
        const ChunkDesc& d = b.desc[c];
        HashView hv;
        hv.prime = st.edge_prime;
        hv.magic = st.edge_magic;
        hv.table = b.edge_slots + st.edge_table_off;
        hv.stash = hv.table + hv.prime;
        hv.stash_used = st.edge_stash_used;
        for (int k = 0; k < 10; k++) hv.p[k] = d.edge_params[k];
        const float4* info = b.edge_info + st.edge_off;
        int x, y, z;
        position_for_code<VPC>(b.node_codes[i], x, y, z);
        const int edge_list = b.node_info[i] >> 16;
        const float fs = (float)d.scale;
        Qef q;
        for (int k = 0; k < 6; k++) q.ata[k] = 0.f;
        q.atb[0] = q.atb[1] = q.atb[2] = 0.f;
        q.mp[0] = q.mp[1] = q.mp[2] = q.mp[3] = 0.f;
        double ata[6] = {0, 0, 0, 0, 0, 0}, atb[3] = {0, 0, 0}, mp[4] = {0, 0, 0, 0};
        for (int e = 0; e < 12; e++) {
            if (!((edge_list >> e) & 1)) continue;
            const int e0 = edge_c0(e), e1 = edge_c1(e);
            const int o0x = e0 >> 2, o0y = (e0 >> 1) & 1, o0z = e0 & 1;
            const int o1x = e1 >> 2, o1y = (e1 >> 1) & 1, o1z = e1 & 1;
            const uint32_t di = hv.find((uint32_t)edge_key<VPC>(x + o0x, y + o0y, z + o0z, e / 4));
            if (di == ~0u) continue;
            const float4 ed = info[di];
            const float p0x = (float)x + (float)o0x, p0y = (float)y + (float)o0y, p0z = (float)z + (float)o0z;
            const float p1x = (float)x + (float)o1x, p1y = (float)y + (float)o1y, p1z = (float)z + (float)o1z;
            const float px = fs * fmaf(p1x - p0x, ed.w, p0x);
            const float py = fs * fmaf(p1y - p0y, ed.w, p0y);
            const float pz = fs * fmaf(p1z - p0z, ed.w, p0z);
            const float pw = fs * fmaf(0.f - 0.f, ed.w, 0.f);
            const float nx = ed.x, ny = ed.y, nzv = ed.z;
            q.ata[0] += nx * nx;
            q.ata[1] += nx * ny;
            q.ata[2] += nx * nzv;
            q.ata[3] += ny * ny;
            q.ata[4] += ny * nzv;
            q.ata[5] += nzv * nzv;
            const float bb = dot4(px, py, pz, pw, nx, ny, nzv, 0.f);
            q.atb[0] += nx * bb;
            q.atb[1] += ny * bb;
            q.atb[2] += nzv * bb;
            q.mp[0] += px;
            q.mp[1] += py;
            q.mp[2] += pz;
            q.mp[3] += 1.f;
            // the same crossing and normal in double
            const double t = ed.w, sd = d.scale;
            const double P[3] = {sd * (p0x + (p1x - p0x) * t), sd * (p0y + (p1y - p0y) * t), sd * (p0z + (p1z - p0z) * t)};
            const double N[3] = {nx, ny, nzv};
            ata[0] += N[0] * N[0];
            ata[1] += N[0] * N[1];
            ata[2] += N[0] * N[2];
            ata[3] += N[1] * N[1];
            ata[4] += N[1] * N[2];
            ata[5] += N[2] * N[2];
            const double bd = P[0] * N[0] + P[1] * N[1] + P[2] * N[2];
            for (int k = 0; k < 3; k++) atb[k] += N[k] * bd;
            for (int k = 0; k < 3; k++) mp[k] += P[k];
            mp[3] += 1.0;
        }
        const float mw = q.mp[3];
        q.mp[0] = q.mp[0] / mw;
        q.mp[1] = q.mp[1] / mw;
        q.mp[2] = q.mp[2] / mw;
        q.mp[3] = q.mp[3] / mw;
        float ox, oy, oz;
        qef_solve(q, ox, oy, oz);
        const float wx = fmaf(ox, (float)LEAF_SIZE_SCALE, (float)d.min[0]);
        const float wy = fmaf(oy, (float)LEAF_SIZE_SCALE, (float)d.min[1]);
        const float wz = fmaf(oz, (float)LEAF_SIZE_SCALE, (float)d.min[2]);
        double o64[3];
        qef_solve_f64(ata, atb, mp, o64);
        const double dx = wx - (o64[0] * LEAF_SIZE_SCALE + d.min[0]);
        const double dy = wy - (o64[1] * LEAF_SIZE_SCALE + d.min[1]);
        const double dz = wz - (o64[2] * LEAF_SIZE_SCALE + d.min[2]);
        const double err = sqrt(dx * dx + dy * dy + dz * dz) / (LEAF_SIZE_SCALE * (double)d.scale);
        if (err == err) {
            local_max = fmax(local_max, err);
            local_sum += err;
            local_n++;
            local_far += err > 1e-3;
        }
    }
    atomicMax(&stats[0], (unsigned long long)__double_as_longlong(local_max));
    atomicAdd(reinterpret_cast<double*>(&stats[1]), local_sum);
    atomicAdd(&stats[2], local_n);
    atomicAdd(&stats[3], local_far);
}

// CreateLeafNodes + SolveQEFs + GenerateMeshVertexBuffer (octree.cl:236-331, 475-487)
template <int VPC, bool HOST>
__global__ void __launch_bounds__(kThreads, 4) k_leaf(BatchPtrs b) {
    if (b.bs->overflow) return;
    const int total = b.bs->total_nodes;
    int lo = 0, hi = total;
    if (b.nslices > 1) {  // this launch's share of the leaves
        lo = (int)((long long)total * b.slice / b.nslices);
        hi = (int)((long long)total * (b.slice + 1) / b.nslices);
    }
    // HOST: the vertices also go to the caller's pinned host array
    // (b.host_vertices) as they are made.  Each warp stages its 32 vertices in
    // shared memory (dynamic, so launches without it keep the whole L1) and
    // writes them as one contiguous run of 16-byte stores, so the C2C traffic
    // starts with the leaves instead of after them; for that the warp walks
    // its 32 consecutive leaves together, lanes past the end idle.  An array
    // too small is not written and the batch is flagged, as k_export does.
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float4* const host = b.host_vertices;
    const bool to_host = HOST && (int64_t)total <= b.host_vertex_cap;
    if (HOST && !to_host && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&b.bs->status, 1);
    extern __shared__ float4 stage_mem[];
    float4* const stage = stage_mem + 96 * wid;
    for (int i0 = lo + blockIdx.x * blockDim.x + (HOST ? (threadIdx.x & ~31) : threadIdx.x); i0 < hi;
         i0 += gridDim.x * blockDim.x) {
      const int i = HOST ? i0 + lane : i0;
      if (!HOST || i < hi) {
        const int c = b.node_chunk[i];
        const ChunkState& st = b.cs[c];
        const ChunkDesc& d = b.desc[c];
        HashView hv;
        hv.prime = st.edge_prime;
        hv.magic = st.edge_magic;
        hv.table = b.edge_slots + st.edge_table_off;
        hv.stash = hv.table + hv.prime;
        hv.stash_used = st.edge_stash_used;
#pragma unroll
        for (int k = 0; k < 10; k++) hv.p[k] = d.edge_params[k];
        const float4* info = b.edge_info + st.edge_off;
        int x, y, z;
        position_for_code<VPC>(b.node_codes[i], x, y, z);
        const int ni = b.node_info[i];
        const int edge_list = ni >> 16;
        const float fs = (float)d.scale;
        Qef q;
#pragma unroll
        for (int k = 0; k < 6; k++) q.ata[k] = 0.f;
        q.atb[0] = q.atb[1] = q.atb[2] = 0.f;
        q.mp[0] = q.mp[1] = q.mp[2] = q.mp[3] = 0.f;
        float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
        const bool simp = b.simp_on != 0;
        SimpQef sq;
        if (simp) simp_zero(sq);
        // every edge lookup first, so that their table probes are in flight
        // together, then the crossings in edge order.  Iteration k handles the
        // leaf's k-th active edge (ascending), so a warp runs as many
        // iterations as its busiest leaf has edges, not one per edge index.
        const int cnt = __popc(edge_list & 0xfff);
        uint32_t dis[12];
        int rest = edge_list & 0xfff;
#pragma unroll
        for (int k = 0; k < 12; k++) {
            if (k >= cnt) break;
            const int e = __ffs(rest) - 1;
            rest &= rest - 1;
            const int e0 = edge_c0(e);
            dis[k] = hv.find((uint32_t)edge_key<VPC>(x + (e0 >> 2), y + ((e0 >> 1) & 1), z + (e0 & 1), e / 4));
        }
        rest = edge_list & 0xfff;
#pragma unroll
        for (int k = 0; k < 12; k++) {
            if (k >= cnt) break;
            const int e = __ffs(rest) - 1;
            rest &= rest - 1;
            const uint32_t di = dis[k];
            if (di == ~0u) continue;
            const int e0 = edge_c0(e), e1 = edge_c1(e);
            const int o0x = e0 >> 2, o0y = (e0 >> 1) & 1, o0z = e0 & 1;
            const int o1x = e1 >> 2, o1y = (e1 >> 1) & 1, o1z = e1 & 1;
            const float4 ed = info[di];
            const float p0x = (float)x + (float)o0x, p0y = (float)y + (float)o0y, p0z = (float)z + (float)o0z;
            const float p1x = (float)x + (float)o1x, p1y = (float)y + (float)o1y, p1z = (float)z + (float)o1z;
            const float px = fs * fmaf(p1x - p0x, ed.w, p0x);
            const float py = fs * fmaf(p1y - p0y, ed.w, p0y);
            const float pz = fs * fmaf(p1z - p0z, ed.w, p0z);
            const float pw = fs * fmaf(0.f - 0.f, ed.w, 0.f);
            // qef_add_point (qef.cl:170-191)
            const float nx = ed.x, ny = ed.y, nzv = ed.z;
            q.ata[0] += nx * nx;
            q.ata[1] += nx * ny;
            q.ata[2] += nx * nzv;
            q.ata[3] += ny * ny;
            q.ata[4] += ny * nzv;
            q.ata[5] += nzv * nzv;
            const float bb = dot4(px, py, pz, pw, nx, ny, nzv, 0.f);
            q.atb[0] += nx * bb;
            q.atb[1] += ny * bb;
            q.atb[2] += nzv * bb;
            q.mp[0] += px;
            q.mp[1] += py;
            q.mp[2] += pz;
            q.mp[3] += 1.f;
            sx += nx;
            sy += ny;
            sz += nzv;
            sw += 1.f;
            if (simp)  // the same crossing in the voxel's own frame
                simp_add_point(sq, fmaf((float)(o1x - o0x), ed.w, (float)o0x), fmaf((float)(o1y - o0y), ed.w, (float)o0y),
                               fmaf((float)(o1z - o0z), ed.w, (float)o0z), nx, ny, nzv);
        }
        if (simp) b.leaf_qef[i] = sq;
        // qef_create_from_points divides the mass point by its count (qef.cl:302)
        const float mw = q.mp[3];
        q.mp[0] = q.mp[0] / mw;
        q.mp[1] = q.mp[1] / mw;
        q.mp[2] = q.mp[2] / mw;
        q.mp[3] = q.mp[3] / mw;
        float ox, oy, oz;
        qef_solve(q, ox, oy, oz);
        lvn_mesh_vertex vtx;
        vtx.position[0] = fmaf(ox, (float)LEAF_SIZE_SCALE, (float)d.min[0]);
        vtx.position[1] = fmaf(oy, (float)LEAF_SIZE_SCALE, (float)d.min[1]);
        vtx.position[2] = fmaf(oz, (float)LEAF_SIZE_SCALE, (float)d.min[2]);
        vtx.position[3] = 1.f;
        vtx.normal[0] = sx / sw;
        vtx.normal[1] = sy / sw;
        vtx.normal[2] = sz / sw;
        vtx.normal[3] = 0.f;
        vtx.colour[0] = d.colour[0];
        vtx.colour[1] = d.colour[1];
        vtx.colour[2] = d.colour[2];
        vtx.colour[3] = (float)((ni & 0xffff) >> 8);
        float4* dst = reinterpret_cast<float4*>((simp ? b.leaf_out : b.vertices) + i);
        const float4 f0 = make_float4(vtx.position[0], vtx.position[1], vtx.position[2], vtx.position[3]);
        const float4 f1 = make_float4(vtx.normal[0], vtx.normal[1], vtx.normal[2], vtx.normal[3]);
        const float4 f2 = make_float4(vtx.colour[0], vtx.colour[1], vtx.colour[2], vtx.colour[3]);
        dst[0] = f0;
        dst[1] = f1;
        dst[2] = f2;
        if (HOST && to_host) {
            stage[3 * lane] = f0;
            stage[3 * lane + 1] = f1;
            stage[3 * lane + 2] = f2;
        }
      }
      if (HOST && to_host) {
        __syncwarp();
        const int n = min(32, hi - i0);
        float4* out = host + 3 * (size_t)i0;
        for (int k = lane; k < 3 * n; k += 32) out[k] = stage[k];
        __syncwarp();
      }
    }
}

// ---------------------------------------------------------------------------
// stage 14-16: quads and seams (GenerateMesh, CompactMeshTriangles,
// FindSeamNodes, ExtractSeamNodeInfo: octree.cl:385-464, 506-551)
// ---------------------------------------------------------------------------

__device__ __forceinline__ int chunk_of_tile(const int* off, int n, int vt) {
    int lo = 0, hi = n;  // largest c in [0, n) with off[c] <= vt
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= vt) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int VPC>
__global__ void __launch_bounds__(kNodeTile) k_mesh_count(BatchPtrs b) {
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int ntiles = b.chunk_tile_off[b.n];
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        int packed = 0;
        if (local < st.nodes) {
            const int i = st.node_off + local;
            HashView hv;
            hv.prime = st.node_prime;
            hv.magic = st.node_magic;
            hv.table = b.node_slots + st.node_table_off;
            hv.stash = hv.table + hv.prime;
            hv.stash_used = st.node_stash_used;
#pragma unroll
            for (int k = 0; k < 10; k++) hv.p[k] = b.desc[c].node_params[k];
            int pos[3];
            position_for_code<VPC>(b.node_codes[i], pos[0], pos[1], pos[2]);
            const int corners = b.node_info[i] & 0xff;
            int quads = 0;
#pragma unroll
            for (int axis = 0; axis < 3; axis++) {
                int4 q = make_int4(-1, -1, -1, 0);
                const int aa = pos[(axis + 1) % 3], bb = pos[(axis + 2) % 3];
                // ProcessEdge (octree.cl:335-372): a quad needs the edge's sign
                // change and all three neighbours; the sign is tested first, so
                // that the neighbour lookups run only for the edges it passes
                const int edge = axis * 4 + 3;
                const int m1 = (corners >> edge_c0(edge)) & 1, m2 = (corners >> edge_c1(edge)) & 1;
                if (aa != VPC - 1 && bb != VPC - 1 && m1 != m2) {
                    // EDGE_NODE_OFFSETS (octree.cl:376-381)
                    int nb[3];
#pragma unroll
                    for (int k = 1; k < 4; k++) {
                        int ox = 0, oy = 0, oz = 0;
                        if (axis == 0) { oy = (k >> 1) & 1; oz = k & 1; }
                        else if (axis == 1) { ox = k & 1; oz = (k >> 1) & 1; }
                        else { oy = k & 1; ox = (k >> 1) & 1; }
                        nb[k - 1] = (int)hv.find(code_for_position<VPC>(pos[0] + ox, pos[1] + oy, pos[2] + oz));
                    }
                    if (nb[0] != -1 && nb[1] != -1 && nb[2] != -1) {
                        q = make_int4(nb[0], nb[1], nb[2], 1 | (m1 != 0 ? 2 : 0));
                        quads++;
                    }
                }
                b.quad_scratch[3 * (size_t)i + axis] = q;
            }
            const bool seam = pos[0] == 0 || pos[0] == VPC - 1 || pos[1] == 0 || pos[1] == VPC - 1 || pos[2] == 0 ||
                              pos[2] == VPC - 1;
            packed = quads | (seam ? 1 << 16 : 0);
        }
        const int total = block_sum<kNodeTile>(packed, sm);
        if (threadIdx.x == 0) b.node_tile_counts[vt] = make_int2(total & 0xffff, total >> 16);
    }
}

__global__ void __launch_bounds__(1024) k_mesh_plan(BatchPtrs b) {
    __shared__ int sm[1024 / 32 + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (b.bs->overflow) return;
    for (int c = warp; c < b.n; c += 32) {
        const int t0 = b.chunk_tile_off[c], nt = b.chunk_tile_off[c + 1] - t0;
        int2* t = b.node_tile_counts + t0;
        int cq = 0, cs = 0;
        for (int base = 0; base < nt; base += 32) {
            const int i = base + lane;
            const int2 v = i < nt ? t[i] : make_int2(0, 0);
            const int iq = warp_inclusive(v.x), is = warp_inclusive(v.y);
            if (i < nt) t[i] = make_int2(cq + iq - v.x, cs + is - v.y);
            cq += __shfl_sync(FULL, iq, 31);
            cs += __shfl_sync(FULL, is, 31);
        }
        if (lane == 0) {
            b.cs[c].quads = cq;
            b.cs[c].seams = cs;
        }
    }
    __syncthreads();
    const long long tq = cta_scan(
        b.n, [&](int c) { return b.cs[c].quads; }, [&](int c, long long ex) { b.cs[c].quad_off = (int)ex; }, nullptr, sm);
    const long long ts = cta_scan(
        b.n, [&](int c) { return b.cs[c].seams; }, [&](int c, long long ex) { b.cs[c].seam_off = (int)ex; }, nullptr, sm);
    if (threadIdx.x == 0) {
        b.bs->total_quads = (int)tq;
        b.bs->total_seams = (int)ts;
        int ovf = 0;
        if (!b.simp_on && 2 * tq > b.triangle_cap) ovf |= OVF_QUADS;  // simplified triangles are checked later
        if (ts > b.seam_cap) ovf |= OVF_SEAMS;
        b.bs->overflow |= ovf;
    }
}

template <int VPC, bool HOST>
__global__ void __launch_bounds__(kNodeTile) k_mesh_scatter(BatchPtrs b) {
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int ntiles = b.chunk_tile_off[b.n];
    // HOST (the seam pass): the seams also go to the caller's pinned host
    // array (b.host_seams).  A tile's seams are contiguous, so the CTA stages
    // them in shared memory (dynamic, this variant only) and writes them as
    // one run of 16-byte stores.  An array too small is not written and the
    // batch is flagged, as k_export does.
    int4* const host = b.host_seams;
    const bool to_host = HOST && (int64_t)b.bs->total_seams <= b.host_seam_cap;
    if (HOST && !to_host && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&b.bs->status, 4);
    extern __shared__ int4 seam_stage[];
    // winding orders by sign-change direction (octree.cl:357-362)
    const int w0[6] = {0, 1, 3, 0, 3, 2};
    const int w1[6] = {0, 3, 1, 0, 2, 3};
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        const bool valid = local < st.nodes;
        const int i = st.node_off + local;
        // the scan packs quads (low 16 bits) and seams (high 16 bits), whose
        // prefixes are independent, so a pass reads only what it writes:
        // scatter_what 1 = triangles, 2 = seams, 0 = both
        int4 q[3] = {make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0)};
        int quads = 0;
        bool seam = false;
        int pos[3] = {0, 0, 0};
        if (valid && b.scatter_what != 2) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                q[a] = b.quad_scratch[3 * (size_t)i + a];
                quads += q[a].w & 1;
            }
        }
        if (valid && b.scatter_what != 1) {
            position_for_code<VPC>(b.node_codes[i], pos[0], pos[1], pos[2]);
            seam = pos[0] == 0 || pos[0] == VPC - 1 || pos[1] == 0 || pos[1] == VPC - 1 || pos[2] == 0 ||
                   pos[2] == VPC - 1;
        }
        int total;
        const int ex = block_exclusive<kNodeTile>(quads | (seam ? 1 << 16 : 0), total, sm);
        if (valid) {
            const int2 toff = b.node_tile_counts[vt];
            int qp = st.quad_off + toff.x + (ex & 0xffff);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (!(q[a].w & 1) || b.simp_on || b.scatter_what == 2) continue;
                const int idx[4] = {local, q[a].x, q[a].y, q[a].z};
                const int* w = (q[a].w & 2) ? w1 : w0;
                lvn_mesh_triangle* tri = b.triangles + 2 * (size_t)qp;
                tri[0].indices[0] = idx[w[0]];
                tri[0].indices[1] = idx[w[1]];
                tri[0].indices[2] = idx[w[2]];
                tri[1].indices[0] = idx[w[3]];
                tri[1].indices[1] = idx[w[4]];
                tri[1].indices[2] = idx[w[5]];
                qp++;
            }
            if (seam && b.scatter_what != 1) {
                const int sp = st.seam_off + toff.y + (ex >> 16);
                const float4* v = reinterpret_cast<const float4*>((b.simp_on ? b.leaf_out : b.vertices) + i);
                int4* dst = reinterpret_cast<int4*>(b.seams + sp);
                const int4 s0 = make_int4(pos[0], pos[1], pos[2], b.node_info[i] & 0xffff);
                const float4 p = v[0], nrm = v[1];
                dst[0] = s0;
                reinterpret_cast<float4*>(dst)[1] = p;
                reinterpret_cast<float4*>(dst)[2] = nrm;
                if (HOST && to_host) {
                    const int r = ex >> 16;
                    seam_stage[3 * r] = s0;
                    reinterpret_cast<float4*>(seam_stage)[3 * r + 1] = p;
                    reinterpret_cast<float4*>(seam_stage)[3 * r + 2] = nrm;
                }
            }
        }
        if (HOST && to_host) {
            __syncthreads();
            const int ns = total >> 16;  // the tile's seams
            if (ns) {
                const ChunkState& tst = b.cs[c];
                int4* out = host + 3 * (size_t)(tst.seam_off + b.node_tile_counts[vt].y);
                for (int k = threadIdx.x; k < 3 * ns; k += blockDim.x) out[k] = seam_stage[k];
            }
            __syncthreads();  // the next tile reuses the staging rows
        }
    }
}


// ---------------------------------------------------------------------------
// Bottom-up octree simplification (not in the reference): classic dual
// contouring collapse (Ju et al. 2002) of each chunk's leaf octree, level by
// level.  A node at level k (2^k voxels) has one entry, created by the first
// of its children to claim its cell in the chunk's level-k grid; it collapses
// when every child that exists collapsed (leaves count, seam voxels do not),
// and its QEF error is at most the threshold.  The mesh keeps GenerateMesh's
// quads (octree.cl:385-442) remapped to each leaf's highest collapsed ancestor
// (its representative): a quad survives on the first sign change along the
// minimal edge (the edge of the smallest of its four representatives) when
// that edge's end points differ in sign, and triangles with a repeated vertex
// are dropped.  Vertices are the representatives, ordered by their first leaf.
// ---------------------------------------------------------------------------

template <int VPC>
__device__ __forceinline__ int simp_grid_off(int k) {  // cells before level k's grid in a chunk
    int s = 0;
    for (int j = 1; j < k; j++) s += (VPC >> j) * (VPC >> j) * (VPC >> j);
    return s;
}

template <int VPC>
__device__ __forceinline__ int* simp_cell(const BatchPtrs& b, int c, int k, int x, int y, int z) {
    const int n = VPC >> k;
    return b.simp_grid + (size_t)c * simp_grid_off<VPC>(Geo<VPC>::DEPTH + 1) + simp_grid_off<VPC>(k) + x +
           n * (y + n * z);
}

// create the level-k entry of cell (x, y, z) of chunk c if it has none
template <int VPC>
__device__ __forceinline__ void simp_claim(const BatchPtrs& b, int c, int k, int x, int y, int z) {
    int* cell = simp_cell<VPC>(b, c, k, x, y, z);
    if (atomicCAS(cell, -1, -2) != -1) return;
    const int e = atomicAdd(b.simp_count + k, 1);
    SimpNode& n = b.simp_nodes[b.simp_level_off[k] + e];
    n.chunk = c;
    n.pos = x | (y << 8) | (z << 16);
    n.collapsed = 0;
    n.anchor = 0;
    atomicExch(cell, e);
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_simp_seed(BatchPtrs b) {
    if (b.bs->overflow) return;
    const int total = b.bs->total_nodes;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int x, y, z;
        position_for_code<VPC>(b.node_codes[i], x, y, z);
        simp_claim<VPC>(b, b.node_chunk[i], 1, x >> 1, y >> 1, z >> 1);
    }
}

template <int VPC>
__global__ void __launch_bounds__(kThreads) k_simp_level(BatchPtrs b, int k) {
    if (b.bs->overflow) return;
    const int count = b.simp_count[k];
    SimpNode* nodes = b.simp_nodes + b.simp_level_off[k];
    const SimpNode* below = b.simp_nodes + b.simp_level_off[k > 1 ? k - 1 : 1];
    const int h = 1 << (k - 1);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
        SimpNode& nd = nodes[e];
        const int c = nd.chunk;
        const int px = nd.pos & 255, py = (nd.pos >> 8) & 255, pz = nd.pos >> 16;
        const ChunkState& st = b.cs[c];
        HashView hv;
        if (k == 1) {
            hv.prime = st.node_prime;
            hv.magic = st.node_magic;
            hv.table = b.node_slots + st.node_table_off;
            hv.stash = hv.table + hv.prime;
            hv.stash_used = st.node_stash_used;
#pragma unroll
            for (int j = 0; j < 10; j++) hv.p[j] = b.desc[c].node_params[j];
        }
        bool blocked = false;
        SimpQef q;
        simp_zero(q);
        int mats[8];
        int anchor = 0x7fffffff;
        for (int i = 0; i < 8; i++) {
            const int ox = (i >> 2) & 1, oy = (i >> 1) & 1, oz = i & 1;  // CHILD_MIN_OFFSETS
            const int cx = 2 * px + ox, cy = 2 * py + oy, cz = 2 * pz + oz;
            mats[i] = MATERIAL_NONE;
            if (blocked) continue;
            if (k == 1) {
                const uint32_t local = hv.find(code_for_position<VPC>(cx, cy, cz));
                if (local == ~0u) continue;
                if (cx == 0 || cx == VPC - 1 || cy == 0 || cy == VPC - 1 || cz == 0 || cz == VPC - 1) {
                    blocked = true;  // seam voxels stay leaves
                    continue;
                }
                const int vi = st.node_off + (int)local;
                simp_merge(q, b.leaf_qef[vi], (float)(ox * h), (float)(oy * h), (float)(oz * h));
                mats[i] = (b.node_info[vi] >> 8) & 0xff;
                anchor = min(anchor, (int)local);
            } else {
                const int ce = *simp_cell<VPC>(b, c, k - 1, cx, cy, cz);
                if (ce < 0) continue;
                const SimpNode& ch = below[ce];
                if (!ch.collapsed) {
                    blocked = true;
                    continue;
                }
                simp_merge(q, ch.q, (float)(ox * h), (float)(oy * h), (float)(oz * h));
                mats[i] = ch.material;
                anchor = min(anchor, ch.anchor);
            }
        }
        int collapsed = 0;
        if (!blocked) {
            float x, y, z;
            const float err = simp_solve(q, (float)(2 * h), x, y, z);
            if (err <= b.simp_threshold) {
                collapsed = 1;
                const ChunkDesc& d = b.desc[c];
                const float fs = (float)d.scale;
                nd.wpos[0] = fmaf(fs * ((float)(px << k) + x), (float)LEAF_SIZE_SCALE, (float)d.min[0]);
                nd.wpos[1] = fmaf(fs * ((float)(py << k) + y), (float)LEAF_SIZE_SCALE, (float)d.min[1]);
                nd.wpos[2] = fmaf(fs * ((float)(pz << k) + z), (float)LEAF_SIZE_SCALE, (float)d.min[2]);
                nd.material = dominant_material(mats);
                nd.anchor = anchor;
                nd.q = q;
            }
        }
        nd.collapsed = collapsed;
        if (k < Geo<VPC>::DEPTH) simp_claim<VPC>(b, c, k + 1, px >> 1, py >> 1, pz >> 1);
    }
}

// each leaf's representative; anchors counted per node tile
template <int VPC>
__global__ void __launch_bounds__(kNodeTile) k_simp_map(BatchPtrs b) {
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int ntiles = b.chunk_tile_off[b.n];
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        int is_anchor = 0;
        if (local < st.nodes) {
            const int i = st.node_off + local;
            int x, y, z;
            position_for_code<VPC>(b.node_codes[i], x, y, z);
            int level = 0, anchor = local, entry = -1;
            for (int k = 1; k <= Geo<VPC>::DEPTH; k++) {
                const int e = *simp_cell<VPC>(b, c, k, x >> k, y >> k, z >> k);
                if (e < 0) break;
                const int64_t ge = b.simp_level_off[k] + e;
                const SimpNode& nd = b.simp_nodes[ge];
                if (!nd.collapsed) break;
                level = k;
                anchor = nd.anchor;
                entry = (int)ge;
            }
            b.simp_rep[i] = anchor | (level << 20);
            b.simp_entry[i] = entry;
            is_anchor = anchor == local ? 1 : 0;
        }
        const int total = block_sum<kNodeTile>(is_anchor, sm);
        if (threadIdx.x == 0) b.simp_tile_counts[vt].x = total;
    }
}

// the triangles each leaf quad keeps
template <int VPC>
__global__ void __launch_bounds__(kNodeTile) k_simp_tcount(BatchPtrs b) {
    using G = Geo<VPC>;
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int w0[6] = {0, 1, 3, 0, 3, 2};
    const int w1[6] = {0, 3, 1, 0, 2, 3};
    const int ntiles = b.chunk_tile_off[b.n];
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        int tris = 0;
        if (local < st.nodes) {
            const int i = st.node_off + local;
            int pos[3];
            position_for_code<VPC>(b.node_codes[i], pos[0], pos[1], pos[2]);
            const uint4* A = plane_ptr<VPC>(b, c, 1);
            const int rep0 = b.simp_rep[i];
            int mask = 0;
            for (int a = 0; a < 3; a++) {
                const int4 q = b.quad_scratch[3 * (size_t)i + a];
                if (!(q.w & 1)) continue;
                const int r[4] = {rep0, b.simp_rep[st.node_off + q.x], b.simp_rep[st.node_off + q.y],
                                  b.simp_rep[st.node_off + q.z]};
                const int minlev = min(min(r[0] >> 20, r[1] >> 20), min(r[2] >> 20, r[3] >> 20));
                if (minlev > 0) {
                    // the minimal edge along axis a through the quad edge's other coordinates
                    const int len = 1 << minlev;
                    int p0[3] = {pos[0], pos[1], pos[2]};
                    p0[(a + 1) % 3] += 1;
                    p0[(a + 2) % 3] += 1;
                    const int s0 = pos[a] & ~(len - 1);
                    auto solid = [&](int t) {
                        int qq[3] = {p0[0], p0[1], p0[2]};
                        qq[a] = t;
                        return !bit4(A[qq[1] + G::FD * qq[2]], qq[0]);
                    };
                    const bool first = solid(s0);
                    bool keep = first != solid(s0 + len);
                    for (int t = s0 + 1; keep && t <= pos[a]; t++) keep = solid(t) == first;
                    if (!keep) continue;
                }
                const int* w = (q.w & 2) ? w1 : w0;
#pragma unroll
                for (int t = 0; t < 2; t++) {
                    const int a0 = r[w[3 * t]] & 0xfffff, a1 = r[w[3 * t + 1]] & 0xfffff, a2 = r[w[3 * t + 2]] & 0xfffff;
                    if (a0 == a1 || a1 == a2 || a0 == a2) continue;
                    mask |= 1 << (2 * a + t);
                    tris++;
                }
            }
            b.simp_mask[i] = (uint8_t)mask;
        }
        const int total = block_sum<kNodeTile>(tris, sm);
        if (threadIdx.x == 0) b.simp_tile_counts[vt].y = total;
    }
}

__global__ void __launch_bounds__(1024) k_simp_plan(BatchPtrs b) {
    __shared__ int sm[1024 / 32 + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (b.bs->overflow) return;
    for (int c = warp; c < b.n; c += 32) {
        const int t0 = b.chunk_tile_off[c], nt = b.chunk_tile_off[c + 1] - t0;
        int2* t = b.simp_tile_counts + t0;
        int cv = 0, ct = 0;
        for (int base = 0; base < nt; base += 32) {
            const int i = base + lane;
            const int2 v = i < nt ? t[i] : make_int2(0, 0);
            const int iv = warp_inclusive(v.x), it = warp_inclusive(v.y);
            if (i < nt) t[i] = make_int2(cv + iv - v.x, ct + it - v.y);
            cv += __shfl_sync(FULL, iv, 31);
            ct += __shfl_sync(FULL, it, 31);
        }
        if (lane == 0) {
            b.cs[c].simp_verts = cv;
            b.cs[c].simp_tris = ct;
        }
    }
    __syncthreads();
    const long long tv = cta_scan(
        b.n, [&](int c) { return b.cs[c].simp_verts; }, [&](int c, long long ex) { b.cs[c].simp_vert_off = (int)ex; },
        nullptr, sm);
    const long long tt = cta_scan(
        b.n, [&](int c) { return b.cs[c].simp_tris; }, [&](int c, long long ex) { b.cs[c].simp_tri_off = (int)ex; },
        nullptr, sm);
    if (threadIdx.x == 0) {
        b.bs->total_simp_verts = (int)tv;
        b.bs->total_simp_tris = (int)tt;
        int ovf = 0;
        if (tt > b.triangle_cap) ovf |= OVF_QUADS;
        if (tv > b.vertex_cap) ovf |= OVF_NODES;
        b.bs->overflow |= ovf;
    }
}

// vertices of the representatives, at their anchors' ranks
template <int VPC>
__global__ void __launch_bounds__(kNodeTile) k_simp_vscatter(BatchPtrs b) {
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int ntiles = b.chunk_tile_off[b.n];
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        const int i = st.node_off + local;
        const bool anchor = local < st.nodes && (b.simp_rep[i] & 0xfffff) == local;
        int total;
        const int ex = block_exclusive<kNodeTile>(anchor ? 1 : 0, total, sm);
        if (anchor) {
            const int ni = b.simp_tile_counts[vt].x + ex;
            b.simp_newidx[i] = ni;
            float4* dst = reinterpret_cast<float4*>(b.vertices + st.simp_vert_off + ni);
            const int entry = b.simp_entry[i];
            if (entry < 0) {
                const float4* src = reinterpret_cast<const float4*>(b.leaf_out + i);
                dst[0] = src[0];
                dst[1] = src[1];
                dst[2] = src[2];
            } else {
                const SimpNode& nd = b.simp_nodes[entry];
                const ChunkDesc& d = b.desc[c];
                dst[0] = make_float4(nd.wpos[0], nd.wpos[1], nd.wpos[2], 1.f);
                dst[1] = make_float4(nd.q.ns[0] / nd.q.w, nd.q.ns[1] / nd.q.w, nd.q.ns[2] / nd.q.w, 0.f);
                dst[2] = make_float4(d.colour[0], d.colour[1], d.colour[2], (float)nd.material);
            }
        }
    }
}

template <int VPC>
__global__ void __launch_bounds__(kNodeTile) k_simp_tscatter(BatchPtrs b) {
    __shared__ int sm[kNodeTile / 32 + 1];
    if (b.bs->overflow) return;
    const int w0[6] = {0, 1, 3, 0, 3, 2};
    const int w1[6] = {0, 3, 1, 0, 2, 3};
    const int ntiles = b.chunk_tile_off[b.n];
    for (int vt = blockIdx.x; vt < ntiles; vt += gridDim.x) {
        const int c = chunk_of_tile(b.chunk_tile_off, b.n, vt);
        const ChunkState& st = b.cs[c];
        const int local = (vt - b.chunk_tile_off[c]) * kNodeTile + threadIdx.x;
        const int i = st.node_off + local;
        const int mask = local < st.nodes ? b.simp_mask[i] : 0;
        int total;
        const int ex = block_exclusive<kNodeTile>(__popc(mask), total, sm);
        if (mask) {
            int tp = st.simp_tri_off + b.simp_tile_counts[vt].y + ex;
            const int rep0 = b.simp_rep[i];
            for (int a = 0; a < 3; a++) {
                if (!((mask >> (2 * a)) & 3)) continue;
                const int4 q = b.quad_scratch[3 * (size_t)i + a];
                const int r[4] = {rep0, b.simp_rep[st.node_off + q.x], b.simp_rep[st.node_off + q.y],
                                  b.simp_rep[st.node_off + q.z]};
                const int* w = (q.w & 2) ? w1 : w0;
                for (int t = 0; t < 2; t++) {
                    if (!((mask >> (2 * a + t)) & 1)) continue;
                    lvn_mesh_triangle* tri = b.triangles + tp++;
#pragma unroll
                    for (int j = 0; j < 3; j++)
                        tri->indices[j] = b.simp_newidx[st.node_off + (r[w[3 * t + j]] & 0xfffff)];
                }
            }
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// export: copy one output pool (vertices, triangles or seams) to the caller's
// array, which may be pinned host memory reached over NVLink-C2C, in 16-byte
// stores.  The element count is read on the device; an array too small is not
// written and the batch is flagged.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_export(BatchPtrs b, int which, void* dst, int64_t capacity) {
    const BatchState& bs = *b.bs;
    if (bs.overflow) return;
    const void* src;
    int64_t count, elem;
    if (which == 0) {
        src = b.vertices;
        count = b.simp_on ? bs.total_simp_verts : bs.total_nodes;
        elem = sizeof(lvn_mesh_vertex);
    } else if (which == 1) {
        src = b.triangles;
        count = b.simp_on ? bs.total_simp_tris : 2 * (int64_t)bs.total_quads;
        elem = sizeof(lvn_mesh_triangle);
    } else {
        src = b.seams;
        count = bs.total_seams;
        elem = sizeof(lvn_seam_node);
    }
    if (count > capacity) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&b.bs->status, 1 << which);
        return;
    }
    // this launch's share: slice `slice` of `nslices` equal element ranges
    int64_t e0 = 0, e1 = count;
    if (b.nslices > 1) {
        e0 = count * b.slice / b.nslices;
        e1 = count * (b.slice + 1) / b.nslices;
    }
    const int64_t b0 = e0 * elem, b1 = e1 * elem;  // byte range, a multiple of 4
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t* s1 = static_cast<const uint32_t*>(src);
    uint32_t* d1 = static_cast<uint32_t*>(dst);
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | (uintptr_t)b0) & 15) == 0) {
        const uint4* s4 = static_cast<const uint4*>(src);
        uint4* d4 = static_cast<uint4*>(dst);
        const int64_t q1 = b1 >> 4;
        for (int64_t i = (b0 >> 4) + t0; i < q1; i += stride) d4[i] = s4[i];
        for (int64_t i = ((q1 << 4) >> 2) + t0; i < (b1 >> 2); i += stride) d1[i] = s1[i];
    } else {
        for (int64_t i = (b0 >> 2) + t0; i < (b1 >> 2); i += stride) d1[i] = s1[i];
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

const char* stage_name(int s) {
    static const char* names[ST_COUNT] = {"field",      "csg",        "edge_count", "edge_plan",   "edge_scatter",
                                          "hermite",    "vox_count",  "vox_plan",   "vox_scatter", "primes", "hash_fill",
                                          "edge_insert", "leaf",      "node_insert", "mesh_count", "mesh_plan",
                                          "mesh_scatter", "simplify"};
    return s >= 0 && s < ST_COUNT ? names[s] : "?";
}

#define LVN_VPC_DISPATCH(VPCVAR, CALL) \
    switch (VPCVAR) {                   \
        case 8: { constexpr int V = 8; CALL; } break;   \
        case 16: { constexpr int V = 16; CALL; } break; \
        case 32: { constexpr int V = 32; CALL; } break; \
        case 64: { constexpr int V = 64; CALL; } break; \
        default: return cudaErrorInvalidValue;          \
    }

// persistent grid of stage `st`: the autotuner's CTAs per SM, else `per_sm`
static inline int persistent_grid(const BatchPtrs& b, int st, int per_sm) {
    return b.num_sms * (b.grid_per_sm[st] > 0 ? b.grid_per_sm[st] : per_sm);
}

cudaError_t launch_reset(const BatchPtrs& b, cudaStream_t s) {
    k_reset<<<(b.n + 255) / 256, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_field(const BatchPtrs& b, cudaStream_t s) {
    dim3 grid(b.vpc + 2, b.n);
    switch (b.density.mode) {
        case LVN_DENSITY_REFERENCE: LVN_VPC_DISPATCH(b.vpc, (k_field<V, LVN_DENSITY_REFERENCE><<<grid, 96, 0, s>>>(b))); break;
        case LVN_DENSITY_FBM2D: LVN_VPC_DISPATCH(b.vpc, (k_field<V, LVN_DENSITY_FBM2D><<<grid, 96, 0, s>>>(b))); break;
        default: LVN_VPC_DISPATCH(b.vpc, (k_field_caves<V><<<grid, 96, 0, s>>>(b))); break;
    }
    if (b.s_on) LVN_VPC_DISPATCH(b.vpc, (k_field_sdens<V><<<grid, 128, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_probe(const BatchPtrs& b, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_probe<V><<<b.n, kProbes, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_gate(const BatchPtrs& b, cudaStream_t s) {
    k_gate<<<b.n, kProbes, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_csg(const BatchPtrs& b, cudaStream_t s) {
    // two CTAs per SM, no more than the batch has pairs
    const int grid = std::max(1, std::min(2 * b.num_sms, b.n * (b.vpc + 2)));
    LVN_VPC_DISPATCH(b.vpc, (k_csg<V><<<grid, dim3(96, kCsgRows), 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_prune_edges(const BatchPtrs& b, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_prune_edges<V><<<1, 1024, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_edge_count(const BatchPtrs& b, cudaStream_t s) {
    dim3 grid(edge_tiles_per_chunk(b.vpc), b.n);
    LVN_VPC_DISPATCH(b.vpc, (k_edge_count<V><<<grid, kThreads, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_edge_plan(const BatchPtrs& b, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_edge_tiles<V><<<(b.n + 7) / 8, 256, 0, s>>>(b)));
    LVN_VPC_DISPATCH(b.vpc, (k_edge_plan<V><<<1, 1024, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_edge_scatter(const BatchPtrs& b, cudaStream_t s) {
    dim3 grid(edge_tiles_per_chunk(b.vpc), b.n);
    LVN_VPC_DISPATCH(b.vpc, (k_edge_scatter<V><<<grid, kThreads, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_hermite(const BatchPtrs& b, cudaStream_t s) {
    const int min_chunks = b.density.mode == LVN_DENSITY_CAVES ? kHermiteSmemMinChunksCaves : kHermiteSmemMinChunks;
    const bool shared_tables = b.hermite_form == 1 || (b.hermite_form == 0 && b.n >= min_chunks);
    if (shared_tables) {
        // the tuned grid in 256-thread units per SM, as for the other stages:
        // 4 units are one 1024-thread CTA per SM, 2 leave half the SMs free
        const int per_sm = b.grid_per_sm[ST_HERMITE] > 0 ? b.grid_per_sm[ST_HERMITE] : 4;
        const int g = std::max(1, b.num_sms * per_sm / (kHermiteSmemThreads / kThreads));
        const int T = kHermiteSmemThreads, smem = kT3Bytes;
        switch (b.density.mode) {
            case LVN_DENSITY_REFERENCE: LVN_VPC_DISPATCH(b.vpc, (k_hermite_smem<V, LVN_DENSITY_REFERENCE><<<g, T, smem, s>>>(b))); break;
            case LVN_DENSITY_FBM2D: LVN_VPC_DISPATCH(b.vpc, (k_hermite_smem<V, LVN_DENSITY_FBM2D><<<g, T, smem, s>>>(b))); break;
            default: LVN_VPC_DISPATCH(b.vpc, (k_hermite_smem<V, LVN_DENSITY_CAVES><<<g, T, smem, s>>>(b))); break;
        }
        return cudaGetLastError();
    }
    const int g = persistent_grid(b, ST_HERMITE, 8);
    switch (b.density.mode) {
        case LVN_DENSITY_REFERENCE: LVN_VPC_DISPATCH(b.vpc, (k_hermite<V, LVN_DENSITY_REFERENCE><<<g, kThreads, 0, s>>>(b))); break;
        case LVN_DENSITY_FBM2D: LVN_VPC_DISPATCH(b.vpc, (k_hermite<V, LVN_DENSITY_FBM2D><<<g, kThreads, 0, s>>>(b))); break;
        default: LVN_VPC_DISPATCH(b.vpc, (k_hermite<V, LVN_DENSITY_CAVES><<<g, kThreads, 0, s>>>(b))); break;
    }
    return cudaGetLastError();
}

// Kernel attributes set once per device: the shared-memory hermite kernels'
// lookup tables are above the default dynamic shared-memory limit.
cudaError_t set_kernel_attributes() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kT3Bytes);
    };
#define LVN_HERMITE_ATTR(V)                                        \
    set((const void*)k_hermite_smem<V, LVN_DENSITY_REFERENCE>);    \
    set((const void*)k_hermite_smem<V, LVN_DENSITY_FBM2D>);        \
    set((const void*)k_hermite_smem<V, LVN_DENSITY_CAVES>);
    LVN_HERMITE_ATTR(8)
    LVN_HERMITE_ATTR(16)
    LVN_HERMITE_ATTR(32)
    LVN_HERMITE_ATTR(64)
#undef LVN_HERMITE_ATTR
    return e;
}

cudaError_t launch_vox_count(const BatchPtrs& b, cudaStream_t s) {
    dim3 grid(vox_tiles_per_chunk(b.vpc), b.n);
    LVN_VPC_DISPATCH(b.vpc, (k_vox_count<V><<<grid, kThreads, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_vox_plan(const BatchPtrs& b, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_vox_plan<V><<<1, 1024, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_vox_scatter(const BatchPtrs& b, cudaStream_t s) {
    dim3 grid(vox_tiles_per_chunk(b.vpc), b.n);
    LVN_VPC_DISPATCH(b.vpc, (k_vox_scatter<V><<<grid, kThreads, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_primes(const BatchPtrs& b, cudaStream_t s) {
    k_primes<<<(b.n + 7) / 8, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_hash_fill(const BatchPtrs& b, cudaStream_t s) {
    k_hash_fill<<<persistent_grid(b, ST_HASH_FILL, 4), 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_edge_insert(const BatchPtrs& b, cudaStream_t s) {
    k_edge_insert<<<persistent_grid(b, ST_EDGE_INSERT, 8), kThreads, 0, s>>>(b);
    k_hash_repair<false><<<(b.n + kRepairThreads - 1) / kRepairThreads, kRepairThreads, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_leaf(const BatchPtrs& b, cudaStream_t s) {
    if (b.host_vertices) {
        LVN_VPC_DISPATCH(b.vpc, (k_leaf<V, true><<<persistent_grid(b, ST_LEAF, 8), kThreads,
                                                   sizeof(float4) * 96 * (kThreads / 32), s>>>(b)));
    } else {
        LVN_VPC_DISPATCH(b.vpc, (k_leaf<V, false><<<persistent_grid(b, ST_LEAF, 8), kThreads, 0, s>>>(b)));
    }
    return cudaGetLastError();
}

cudaError_t launch_node_insert(const BatchPtrs& b, cudaStream_t s) {
    k_node_insert<<<persistent_grid(b, ST_NODE_INSERT, 8), kThreads, 0, s>>>(b);
    k_hash_repair<true><<<(b.n + kRepairThreads - 1) / kRepairThreads, kRepairThreads, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_mesh_count(const BatchPtrs& b, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_mesh_count<V><<<persistent_grid(b, ST_MESH_COUNT, 8), kNodeTile, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_simplify(const BatchPtrs& b, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(b.simp_grid, 0xff, sizeof(int) * (size_t)b.n * (size_t)simp_grid_cells(b.vpc), s);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b.simp_count, 0, sizeof(int) * 8, s)) != cudaSuccess) return e;
    const int g = persistent_grid(b, ST_SIMPLIFY, 8);
    LVN_VPC_DISPATCH(b.vpc, (k_simp_seed<V><<<g, kThreads, 0, s>>>(b)));
    for (int k = 1; k <= octree_depth(b.vpc); k++) LVN_VPC_DISPATCH(b.vpc, (k_simp_level<V><<<g, kThreads, 0, s>>>(b, k)));
    LVN_VPC_DISPATCH(b.vpc, (k_simp_map<V><<<g, kNodeTile, 0, s>>>(b)));
    LVN_VPC_DISPATCH(b.vpc, (k_simp_tcount<V><<<g, kNodeTile, 0, s>>>(b)));
    k_simp_plan<<<1, 1024, 0, s>>>(b);
    LVN_VPC_DISPATCH(b.vpc, (k_simp_vscatter<V><<<g, kNodeTile, 0, s>>>(b)));
    LVN_VPC_DISPATCH(b.vpc, (k_simp_tscatter<V><<<g, kNodeTile, 0, s>>>(b)));
    return cudaGetLastError();
}

cudaError_t launch_mesh_plan(const BatchPtrs& b, cudaStream_t s) {
    k_mesh_plan<<<1, 1024, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_export(const BatchPtrs& b, int which, void* dst, int64_t capacity, cudaStream_t s) {
    k_export<<<b.num_sms, 256, 0, s>>>(b, which, dst, capacity);  // one CTA per SM saturates C2C
    return cudaGetLastError();
}

cudaError_t launch_mesh_scatter(const BatchPtrs& b, cudaStream_t s) {
    if (b.host_seams) {
        LVN_VPC_DISPATCH(b.vpc, (k_mesh_scatter<V, true><<<persistent_grid(b, ST_MESH_SCATTER, 8), kNodeTile,
                                                          sizeof(int4) * 3 * kNodeTile, s>>>(b)));
    } else {
        LVN_VPC_DISPATCH(b.vpc, (k_mesh_scatter<V, false><<<persistent_grid(b, ST_MESH_SCATTER, 8), kNodeTile, 0,
                                                           s>>>(b)));
    }
    return cudaGetLastError();
}

cudaError_t launch_debug_cuckoo(const uint32_t* keys, int n, unsigned long long* table, uint32_t prime,
                                CuckooParams params, int* status, int reference_find, uint32_t* values,
                                cudaStream_t s) {
    if (n <= 0 || prime < 2) return cudaErrorInvalidValue;
    const uint32_t magic = 0xffffffffu / prime;
    const int64_t slots = (int64_t)prime + CUCKOO_STASH_SIZE;
    k_debug_cuckoo_fill<<<(int)std::min<int64_t>((slots + 255) / 256, 1024), 256, 0, s>>>(table, slots);
    const int grid = std::min((n + 255) / 256, 1024);
    k_debug_cuckoo_insert<<<grid, 256, 0, s>>>(keys, n, table, prime, magic, params, status);
    k_debug_cuckoo_find<<<grid, 256, 0, s>>>(keys, n, table, prime, magic, params, status, reference_find, values);
    return cudaGetLastError();
}

cudaError_t launch_leaf_qef_check(const BatchPtrs& b, unsigned long long* stats, cudaStream_t s) {
    LVN_VPC_DISPATCH(b.vpc, (k_leaf_qef_check<V><<<b.num_sms * 4, 256, 0, s>>>(b, stats)));
    return cudaGetLastError();
}

}  // namespace lvn
