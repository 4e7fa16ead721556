// lvn_surrogate.cu -- learned density surrogate (not in the reference).
//
// A multilayer perceptron from a density-space position to the density:
//   16 frequencies per axis, sin and cos (96 Fourier features)
//   -> 4 x [Linear 128, SiLU] -> Linear 1
// 62,081 parameters.  Weights and activations are BF16, every product is
// accumulated in FP32, the master weights and Adam moments are FP32.
//
// Every matrix product runs on the 5th-generation tensor cores (tcgen05.mma,
// kind::f16: BF16 in, FP32 accumulator in tensor memory), issued by one thread
// per CTA on 128-row tiles staged in shared memory, with bounded waits on the
// MMA's mbarrier commit:
//   * training (k_mlp_train): one persistent kernel a step for the features,
//     the forward, the loss, the backward and every gradient; Adam on the CUDA
//     cores (k_adam_partials);
//   * inference (k_mlp_infer): the whole network per 128-point tile.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/lvn.h"
#include "lvn_noise.cuh"
#include "lvn_state.h"

namespace lvn {
namespace {

constexpr int kHidden = 128;
constexpr int kFreqs = 16;
constexpr int kIn = 6 * kFreqs;  // 96
constexpr int kLayers = 4;       // hidden layers
constexpr int kTile = 128;       // rows per CTA tile (MMA M)
constexpr uint32_t kWaitLimit = 1u << 20;  // mbarrier polls before a CTA gives up

// parameter offsets in the flat FP32 vector: W0 b0 W1 b1 W2 b2 W3 b3 w4 b4
constexpr int kIn_[kLayers] = {kIn, kHidden, kHidden, kHidden};
__host__ __device__ constexpr int in_dim(int l) { return l == 0 ? kIn : kHidden; }
// (closed forms: the kernels also call these with run-time layer indices)
__host__ __device__ constexpr int w_off(int l) {
    return l == 0 ? 0 : (kHidden * kIn + kHidden) + (l - 1) * (kHidden * kHidden + kHidden);
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + kHidden * in_dim(l); }
constexpr int kHeadW = w_off(kLayers);
constexpr int kHeadB = kHeadW + kHidden;
constexpr int kParams = kHeadB + 1;
static_assert(w_off(2) == w_off(1) + kHidden * kHidden + kHidden && b_off(0) == kHidden * kIn, "layout");
static_assert(kParams == 62081, "4 x 128 SiLU MLP on 96 features");
// BF16 copies W_l (out x in)
__host__ __device__ constexpr int wb_off(int l) { return l == 0 ? 0 : kHidden * kIn + (l - 1) * kHidden * kHidden; }
constexpr int kWb = wb_off(kLayers);

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier primitives (inline PTX, sm_100 family)
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.b32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// UMMA shared-memory descriptor, K-major without swizzle: core matrices of
// 8 rows x 16 bytes; `lbo` = bytes between core matrices along K, `sbo` =
// bytes between core matrices along M / N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of the tcgen05 family; base offset 0, no swizzle
    return d;
}
// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// A chain of STEPS MMAs over K = 16 STEPS: the descriptors' start addresses
// advance by a_step / b_step bytes a step (an immediate add to the low word:
// shared-memory addresses are below 256 KB, so the 14-bit field never
// carries).  The first MMA overwrites D unless `acc`.
template <int STEPS>
__device__ __forceinline__ void umma_chain(uint32_t tmem_d, uint64_t adesc, uint32_t a_step, uint64_t bdesc,
                                           uint32_t b_step, uint32_t idesc, bool acc) {
    const uint32_t alo = (uint32_t)adesc, ahi = (uint32_t)(adesc >> 32);
    const uint32_t blo = (uint32_t)bdesc, bhi = (uint32_t)(bdesc >> 32);
#pragma unroll
    for (int s = 0; s < STEPS; s++) {
        const uint32_t c = (acc || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\n.reg .b64 da, db;\nsetp.ne.b32 p, %6, 0;\nmov.b64 da, {%1, %2};\nmov.b64 db, {%3, %4};\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %5, p;\n}" ::"r"(tmem_d),
            "r"(alo + (uint32_t)s * (a_step >> 4)), "r"(ahi), "r"(blo + (uint32_t)s * (b_step >> 4)), "r"(bhi), "r"(idesc),
            "r"(c)
            : "memory");
    }
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16-byte global -> shared copies that stay in flight together
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// SiLU through sigmoid(z) = (1 + tanh(z / 2)) / 2: one special-function
// instruction (tanh.approx, relative error about 2^-11, below BF16's 2^-8)
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
// the same on two values at once: the FP32 arithmetic in the two-lane forms
// (one instruction for both), the hyperbolic tangent per lane
__device__ __forceinline__ float2 sigmoid2(float2 z) {
    const float2 h = mul2(z, v2(0.5f));
    return fma2(v2(0.5f), make_float2(tanh_approx(h.x), tanh_approx(h.y)), v2(0.5f));
}
__device__ __forceinline__ float2 silu_grad2(float2 z, float2 s) {  // s = sigmoid2(z)
    return mul2(s, fma2(z, sub2(v2(1.f), s), v2(1.f)));
}
// sin(pi r), cos(pi r): r reduced to [-1, 1] exactly (an even number of half
// turns removed), then the fast intrinsics on a small argument
__device__ __forceinline__ void sincos_pi(float r, float& s, float& c) {
    r -= 2.f * rintf(0.5f * r);
    __sincosf(3.14159265358979f * r, &s, &c);
}

// ---------------------------------------------------------------------------
// CUDA-core kernels: training samples, the BF16 weight copies
// ---------------------------------------------------------------------------

struct Domain {
    float lo[3], hi[3];
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ float unit(uint64_t h) { return (float)(h >> 40) * (1.f / 16777216.f); }

// 70% of the samples within 4 voxels of the heightfield surface (y = amp h +
// U(-4, 4), so |d| <= 4 for the heightfield), 30% uniform in the domain;
// target = the plain density.
// 70% within 4 voxels of the zero set, 30% uniform in the domain.  Without a
// 3D term the zero set is the height surface, y = amp h(x, z) + U(-4, 4).
// With one (caves), the zero set lies within `band` of that surface: up to
// eight heights y = amp h + U(-band - 4, band + 4) are tried and the first
// with |density| <= 4 is kept (else the last).
__global__ void k_samples(float4* out, int n, uint64_t seed, Domain dom, const uint8_t* perm_t3,
                          const float* grad, DensityParams dp, float band) {
    __shared__ __align__(16) float sg[64];
    stage_gradients(sg, grad);
    __syncthreads();
    const Noise nz{perm_t3, sg};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t h0 = mix64(seed ^ mix64((uint64_t)i * 4 + 0)), h1 = mix64(seed ^ mix64((uint64_t)i * 4 + 1));
        const uint64_t h2 = mix64(seed ^ mix64((uint64_t)i * 4 + 2)), h3 = mix64(seed ^ mix64((uint64_t)i * 4 + 3));
        const float x = dom.lo[0] + unit(h1) * (dom.hi[0] - dom.lo[0]);
        const float z = dom.lo[2] + unit(h2) * (dom.hi[2] - dom.lo[2]);
        float y, d;
        if (unit(h0) < 0.7f) {
            const float surf = nz.height_amp(dp) * nz.height(dp, x, z);
            if (band > 0.f) {
                uint64_t h = h3;
                for (int k = 0; k < 8; k++) {
                    y = surf + (unit(h) * 2.f - 1.f) * (band + 4.f);
                    d = nz.density(dp, x, y, z);
                    if (fabsf(d) <= 4.f) break;
                    h = mix64(h ^ 0x9E3779B97F4A7C15ull);
                }
            } else {
                y = surf + (unit(h3) * 8.f - 4.f);
                d = nz.density(dp, x, y, z);
            }
        } else {
            y = dom.lo[1] + unit(h3) * (dom.hi[1] - dom.lo[1]);
            d = nz.density(dp, x, y, z);
        }
        out[i] = make_float4(x, y, z, d);
    }
}

struct FeatureFreqs {
    float f[3][kFreqs];
};

struct LayerMap {
    int w[kLayers], b[kLayers], in[kLayers], wb[kLayers];
};

// the BF16 copies W_l (out x in, row-major) of the FP32 hidden weights
__global__ void k_to_bf16(const float* p, int n, __nv_bfloat16* wb, LayerMap lm) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int l = 0; l < kLayers; l++) {
            const int rel = i - lm.w[l];
            if (rel >= 0 && rel < kHidden * lm.in[l]) wb[lm.wb[l] + rel] = __float2bfloat16_rn(p[i]);
        }
    }
}

// ---------------------------------------------------------------------------
// Fused inference: the whole network on 128-point tiles in one CTA.  The four
// hidden layers' BF16 weights stay in shared memory for the kernel's life.
// Three warpgroups each own a tile stream, a 128-column TMEM accumulator and an
// activation tile: a warpgroup computes its tile's features into the tile,
// its elected thread issues the layer's MMAs and commits to its mbarrier, and
// its epilogue turns the accumulator into the next layer's operand (bias,
// SiLU, BF16) in place, or into the density after the last layer.  While one
// warpgroup is in an epilogue the tensor core works on the other's layer.
// ---------------------------------------------------------------------------

constexpr int kWbBytes = 2 * kWb;                 // 120 KB of weights
constexpr int kActBytes = kTile * kHidden * 2;    // 32 KB per activation tile
constexpr int kInferWG = 3;                       // warpgroups (tile streams) per CTA
constexpr int kInferSmem = kWbBytes + kInferWG * kActBytes + (kLayers * kHidden + kHidden + 1) * 4;
static_assert(kInferSmem <= 227 * 1024, "one CTA per SM");

struct InferArgs {
    const float4* pts;       // points (x, y, z, -), or
    const float4* lattices;  // when not null: lattices (x0, y0, z0, step) of dim^3 points, x fastest
    int dim;
    int64_t n;
    const __nv_bfloat16* wb;
    const float* params;
    Domain dom;
    FeatureFreqs ff;
    float out_scale;
    float* out;
    int* status;
};

__device__ __forceinline__ void wg_sync(int wg) {  // named barrier of one warpgroup
    asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory");
}
// named barrier of one warpgroup that also ORs a predicate across it
__device__ __forceinline__ bool wg_any(int wg, bool v) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\nselp.u32 %0, 1, 0, q;\n}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + wg)
        : "memory");
    return r != 0;
}

__global__ void __launch_bounds__(128 * kInferWG, 1) k_mlp_infer(InferArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bars[kInferWG];
    __shared__ uint32_t tmem_base;
    uint8_t* sW = smem;
    uint8_t* sAct = smem + kWbBytes;
    float* sBias = reinterpret_cast<float*>(sAct + kInferWG * kActBytes);  // [4][128] biases, w4[128], b4
    const int warp = threadIdx.x >> 5;
    const int wg = warp >> 2;
    const int row = threadIdx.x & 127;  // tile row = TMEM lane
    // weights: layer l is N = 128 rows (out) x K = in_l, K-major core matrices
    constexpr uint32_t kLbo = (kTile / 8) * 128;  // 2048: 128 rows per K column of core matrices
    for (int l = 0; l < kLayers; l++) {
        const int in = in_dim(l), cores = in / 8;
        uint8_t* dst = sW + 2 * wb_off(l);
        for (int i = threadIdx.x; i < kHidden * cores; i += blockDim.x) {
            const int r = i % kHidden, c = i / kHidden;
            cp_async16(dst + c * kLbo + r * 16, a.wb + wb_off(l) + (size_t)r * in + 8 * c);
        }
    }
    for (int i = threadIdx.x; i < kLayers * kHidden; i += blockDim.x)
        sBias[i] = a.params[b_off(i / kHidden) + (i % kHidden)];
    for (int i = threadIdx.x; i <= kHidden; i += blockDim.x) sBias[kLayers * kHidden + i] = a.params[kHeadW + i];
    if (warp == 0) tmem_alloc(&tmem_base, 512);  // a power of two >= 128 per warpgroup
    if (threadIdx.x < kInferWG) mbar_init(&bars[threadIdx.x], 1);
    cp_async_wait_all();
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base + (uint32_t)(wg * kHidden);  // this warpgroup's columns
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint8_t* act = sAct + wg * kActBytes;
    const uint32_t act_addr = smem_u32(act), w_addr = smem_u32(sW);
    const float* w4 = sBias + kLayers * kHidden;
    const float b4 = w4[kHidden];
    constexpr uint32_t kIdesc = umma_idesc(kTile, kHidden);
    uint32_t phase = 0;
    bool ok = true;
    const int64_t ntiles = (a.n + kTile - 1) / kTile;
    const int64_t per = (int64_t)a.dim * a.dim * a.dim;
    for (int64_t t = (int64_t)blockIdx.x * kInferWG + wg; t < ntiles && ok; t += (int64_t)gridDim.x * kInferWG) {
        const int64_t p = t * kTile + row;
        float c[3] = {0.f, 0.f, 0.f};
        if (p < a.n) {
            if (a.lattices) {
                const int64_t l = p / per;
                const int r = (int)(p - l * per);
                const float4 o = a.lattices[l];
                c[0] = o.x + o.w * (float)(r % a.dim);
                c[1] = o.y + o.w * (float)((r / a.dim) % a.dim);
                c[2] = o.z + o.w * (float)(r / (a.dim * a.dim));
            } else {
                const float4 q = a.pts[p];
                c[0] = q.x;
                c[1] = q.y;
                c[2] = q.z;
            }
        }
        // Above and below the domain's y range the density is extrapolated
        // with unit slope from the range's edge (d = y - h(x, z) + caves has
        // slope 1 away from the surface band), so tall coarse chunks whose
        // surface lies inside the range keep the right sign everywhere.
        const float yc = fminf(fmaxf(c[1], a.dom.lo[1]), a.dom.hi[1]);
        const float y_out = c[1] - yc;
        c[1] = yc;
        // features -> this row of the activation tile (12 core-matrix columns)
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const float u = 2.f * (c[ax] - a.dom.lo[ax]) / (a.dom.hi[ax] - a.dom.lo[ax]) - 1.f;
            __align__(16) __nv_bfloat16 sv[16], cv[16];
#pragma unroll
            for (int k = 0; k < kFreqs; k++) {
                float s, co;
                sincos_pi(a.ff.f[ax][k] * u, s, co);
                sv[k] = __float2bfloat16_rn(s);
                cv[k] = __float2bfloat16_rn(co);
            }
            const int c0 = ax * 4;  // 32 features = 4 core columns per axis
            *reinterpret_cast<uint4*>(act + (c0 + 0) * kLbo + row * 16) = *reinterpret_cast<uint4*>(sv);
            *reinterpret_cast<uint4*>(act + (c0 + 1) * kLbo + row * 16) = *reinterpret_cast<uint4*>(sv + 8);
            *reinterpret_cast<uint4*>(act + (c0 + 2) * kLbo + row * 16) = *reinterpret_cast<uint4*>(cv);
            *reinterpret_cast<uint4*>(act + (c0 + 3) * kLbo + row * 16) = *reinterpret_cast<uint4*>(cv + 8);
        }
        float y = b4;
        for (int l = 0; l < kLayers && ok; l++) {
            fence_proxy_async();
            tc_fence_before();
            wg_sync(wg);
            tc_fence_after();
            if (row == 0) {
                const uint64_t ad = umma_desc(act_addr, kLbo, 128), bd = umma_desc(w_addr + 2 * wb_off(l), kLbo, 128);
                if (l == 0) umma_chain<kIn / 16>(tmem, ad, 2 * kLbo, bd, 2 * kLbo, kIdesc, false);
                else umma_chain<kHidden / 16>(tmem, ad, 2 * kLbo, bd, 2 * kLbo, kIdesc, false);
                umma_commit(&bars[wg]);
            }
            uint32_t polls = 0;
            bool late = false;
            while (!mbar_try_wait(&bars[wg], phase))
                if (++polls == kWaitLimit) {
                    late = true;
                    break;
                }
            phase ^= 1u;
            ok = !wg_any(wg, late);  // the whole warpgroup takes the same path
            tc_fence_after();
            if (!ok) break;
            const float* bias = sBias + l * kHidden;
#pragma unroll 1
            for (int cc = 0; cc < kHidden / 32; cc++) {
                float v[32];
                tmem_ld32(tmem + lane_base + (uint32_t)(cc * 32), v);
                if (l < kLayers - 1) {
                    __align__(16) __nv_bfloat16 h[32];
#pragma unroll
                    for (int j = 0; j < 32; j++) h[j] = __float2bfloat16_rn(silu(v[j] + bias[cc * 32 + j]));
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        *reinterpret_cast<uint4*>(act + (cc * 4 + q) * kLbo + row * 16) =
                            *reinterpret_cast<uint4*>(h + 8 * q);
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        // the head reads the BF16 activation, as in training
                        const float x = __bfloat162float(__float2bfloat16_rn(silu(v[j] + bias[cc * 32 + j])));
                        y = fmaf(x, w4[cc * 32 + j], y);
                    }
                }
            }
        }
        if (ok && p < a.n) a.out[p] = fmaf(y, a.out_scale, y_out);
    }
    if (!ok) {
        // The MMAs this warpgroup committed did not signal within the poll
        // limit.  TMEM is freed below, and a later CTA on this SM may allocate
        // the same columns, so first wait (bounded again) for the commit:
        // once it arrives the MMAs are complete and nothing writes the
        // columns.  If it still does not, the columns are freed all the same
        // (a CTA that never frees them would stall every later allocation on
        // this SM), and the status flag makes the host discard the call's
        // results (LVN_ERR_DEVICE_STATUS), including anything a late MMA wrote.
        if ((threadIdx.x & 127) == 0) atomicExch(a.status, 1);
        uint32_t polls = 0;
        while (!mbar_try_wait(&bars[wg], phase ^ 1u) && ++polls < 4 * kWaitLimit) {
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem_base, 512);
}

// ---------------------------------------------------------------------------
// Fused training: the forward, the loss, the backward and the weight and bias
// gradients of 128-row tiles in one persistent kernel, one launch per step.
//
// Each CTA (16 warps) takes a run of tiles.  The four hidden layers' BF16
// weights stay in shared memory, with two activation images, one dZ image and
// a 128 x 16 image of ones (220 KB).  A thread owns TMEM lane / tile row
// 32 (warp & 3) + lane and the 32-column chunk 32 (warp >> 2) .. + 31.
//
// Per tile:
//   features -> XA (and the X0 image to the tile's slot in scratch)
//   layer l: acc = X_l W_l^T; z = acc + b_l -> BF16 z image (scratch);
//            X_{l+1} = BF16 silu(z) -> the other image (X1 also to the slot)
//   head:    y = X4 . w4 + b4 (four chunk sums), r = y - t / s, dy = 2 r / n,
//            dZ3 = dy w4 silu'(z3) -> the dZ image
//   l = 3, 2: dW_l += dZ_l^T X_l, db_l += dZ_l^T 1 and acc = dZ_l W_l in one
//            commit; dZ_{l-1} = acc silu'(z_{l-1}) -> the dZ image (dZ1 also
//            to the slot)
//   l = 1:   acc = dZ1 W1; dZ0 = acc silu'(z0) -> the slot
// dW_3, dW_2 and their bias sums accumulate in tensor memory over the CTA's
// tiles.  After the last tile they are written out and the freed columns take
// dW_1, dW_0 and their bias sums, contracted from the slots' X1 / dZ1 and
// X0 / dZ0 images (about 480 KB of scratch per CTA, in L2).
//
// The weight-gradient products read the dZ and X images as MN-major operands
// (the same core matrices, K running over the tile's rows) and the input
// gradient reads W_l as an MN-major B, so no transposed copy is made.  A bias
// gradient is the product of dZ^T with the ones image (column 0 of 16 kept).
// The head's weight gradient is a column sum over rows on the CUDA cores (a
// butterfly that leaves column L's sum of a warp's rows in lane L).  The CTA
// writes its gradient and loss to its own row of `partial`; k_adam_partials
// sums the rows in a fixed order, so a step is deterministic.
// ---------------------------------------------------------------------------

constexpr uint32_t kCoreCol = (kTile / 8) * 128;  // bytes between core-matrix columns of a 128-row image
constexpr int kTrainThreads = 512;  // 16 warps: lane quarter warp & 3, column quarter warp >> 2
constexpr int kX0Bytes = kTile * kIn * 2;       // 24 KB feature image
constexpr int kImgBytes = kTile * kHidden * 2;  // 32 KB activation image
constexpr int kOnesBytes = kTile * 16 * 2;      // 4 KB: 128 rows x 16 columns of 1.0
constexpr int kTrainSmem = kWbBytes + 3 * kImgBytes + kOnesBytes;
static_assert(kTrainSmem + 4 * kTile * 4 + 64 <= 227 * 1024, "one CTA per SM");
// per tile slot: the X0, X1, dZ0 and dZ1 images, contracted after the last tile
constexpr size_t kSlotBytes = (size_t)kX0Bytes + 3 * (size_t)kImgBytes;
constexpr size_t kTransientBytes = 3 * (size_t)kImgBytes;  // z0, z1, z2 of the tile in hand
constexpr int kPartStride = (kParams + 1 + 3) / 4 * 4;     // gradient, then the loss; 16-byte rows
// tensor-memory columns
constexpr uint32_t kTmWork = 0;    // forward and input-gradient accumulator
constexpr uint32_t kTmDW2 = 128;   // dW_2 over the CTA's tiles; dW_1 after the last tile
constexpr uint32_t kTmDW3 = 256;   // dW_3; dW_0 (96 columns) after the last tile
constexpr uint32_t kTmDB = 384;    // db_2 / db_1 (16 columns), then db_3 / db_0 (16 columns)
constexpr uint32_t kIdescFwd = umma_idesc(kTile, kHidden);
constexpr uint32_t kIdescDX = umma_idesc(kTile, kHidden) | (1u << 16);                 // B MN-major
constexpr uint32_t kIdescDW = umma_idesc(kHidden, kHidden) | (1u << 15) | (1u << 16);  // A and B MN-major
constexpr uint32_t kIdescDW0 = umma_idesc(kHidden, kIn) | (1u << 15) | (1u << 16);
constexpr uint32_t kIdescDB = umma_idesc(kHidden, 16) | (1u << 15) | (1u << 16);

struct TrainArgs {
    const float4* pool;  // samples (x, y, z, density); row i of the batch is pool[(first + i) % pool_n]
    int64_t pool_n, first;
    int n;               // batch rows, a multiple of kTile
    int tiles_per_cta;
    const __nv_bfloat16* wb;
    const float* params;
    Domain dom;
    FeatureFreqs ff;
    float out_scale;
    uint8_t* scratch;  // gridDim.x x (tiles_per_cta x kSlotBytes + kTransientBytes)
    float* partial;    // gridDim.x x kPartStride
    int* status;
};

// byte offset of core-matrix column c (8 elements), row r of a 128-row image
__device__ __forceinline__ uint32_t img_off(int c, int r) { return (uint32_t)c * kCoreCol + (uint32_t)r * 16u; }

__device__ __forceinline__ uint32_t bf2_bits(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ uint4 pack8(const float* v) {
    return make_uint4(bf2_bits(v[0], v[1]), bf2_bits(v[2], v[3]), bf2_bits(v[4], v[5]), bf2_bits(v[6], v[7]));
}
__device__ __forceinline__ void unpack8(uint4 u, float* v) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[i]));
        v[2 * i] = f.x;
        v[2 * i + 1] = f.y;
    }
}

// Column sums of a warp's 32 rows: lane L holds row L's 32 values in v (which
// this overwrites) and gets back the sum of column L over the 32 rows.  Each
// of the five halvings keeps half of the remaining columns and adds the
// partner lane's copy of them (31 shuffles in all).
__device__ __forceinline__ float warp_column_sums(float (&v)[32], int lane) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < off; j++) {
            const float send = up ? v[j] : v[j + off];
            const float keep = up ? v[j + off] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

// every thread waits for the commit; false for the whole CTA when it did not
// arrive within the poll limit
__device__ __forceinline__ bool cta_wait(uint64_t* bar, uint32_t& phase) {
    uint32_t polls = 0;
    bool late = false;
    while (!mbar_try_wait(bar, phase))
        if (++polls == kWaitLimit) {
            late = true;
            break;
        }
    phase ^= 1u;
    const bool ok = !__syncthreads_or(late);
    tc_fence_after();
    return ok;
}

// shared-memory writes of this CTA made visible to the tensor core, then one
// barrier; thread 0 issues next
__device__ __forceinline__ void to_tensor_core() {
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
}

// 32 consecutive floats (16-byte aligned, the same for every lane) into registers
__device__ __forceinline__ void load32(const float* p, float (&v)[32]) {
    const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const float4 t = __ldg(p4 + i);
        v[4 * i] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

__global__ void __launch_bounds__(kTrainThreads, 1) k_mlp_train(TrainArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ float ypart[4][kTile];
    uint8_t* sW = smem;
    uint8_t* sXA = smem + kWbBytes;
    uint8_t* sXB = sXA + kImgBytes;
    uint8_t* sDZ = sXB + kImgBytes;
    uint8_t* sOnes = sDZ + kImgBytes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = warp & 3, cq = warp >> 2;
    const int row = 32 * q + lane;  // tile row = TMEM lane; columns 32 cq .. 32 cq + 31
    const uint32_t tl = ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * cq);  // this thread's lane and chunk
    for (int l = 0; l < kLayers; l++) {
        const int in = in_dim(l), cores = in / 8;
        uint8_t* dst = sW + 2 * wb_off(l);
        for (int i = threadIdx.x; i < kHidden * cores; i += blockDim.x) {
            const int r = i % kHidden, c = i / kHidden;
            cp_async16(dst + img_off(c, r), a.wb + wb_off(l) + (size_t)r * in + 8 * c);
        }
    }
    for (int i = threadIdx.x; i < kOnesBytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(sOnes)[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    if (warp == 0) tmem_alloc(&tmem_base, 512);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    cp_async_wait_all();
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t w_addr = smem_u32(sW), xa_addr = smem_u32(sXA), xb_addr = smem_u32(sXB), dz_addr = smem_u32(sDZ);
    const uint32_t ones_addr = smem_u32(sOnes);
    uint8_t* scr = a.scratch + (size_t)blockIdx.x * ((size_t)a.tiles_per_cta * kSlotBytes + kTransientBytes);
    auto zimg = [scr](int l) { return scr + (size_t)l * kImgBytes; };  // z_l, l = 0, 1, 2
    uint8_t* slots = scr + kTransientBytes;  // per tile: X0, X1, dZ0, dZ1
    const int ntiles = a.n / kTile;
    const int t0 = blockIdx.x * a.tiles_per_cta, t1 = min(ntiles, t0 + a.tiles_per_cta);
    const float b4 = a.params[kHeadB];
    float gw4 = 0.f, lsum = 0.f, gb4 = 0.f;  // w4 column 32 cq + lane over the warp's rows; loss and b4 per row
    uint32_t phase = 0;
    bool ok = true;
    // dW_l (+)= dZ^T X over one tile's rows (M = 128 outputs, N = `n_in` inputs,
    // both operands MN-major) and db_l (+)= dZ^T 1, issued by thread 0
    const uint64_t dz_mn = umma_desc(dz_addr, 128, kCoreCol), ones_mn = umma_desc(ones_addr, 128, kCoreCol);
    auto weight_grads = [&](uint32_t dw, uint32_t db, uint32_t x_addr, uint32_t idesc, bool acc) {
        umma_chain<kTile / 16>(tmem + dw, dz_mn, 256, umma_desc(x_addr, 128, kCoreCol), 256, idesc, acc);
        umma_chain<kTile / 16>(tmem + db, dz_mn, 256, ones_mn, 256, kIdescDB, acc);
    };
    // the features of tile t -> XA and its slot's X0 image; its targets
    auto features = [&](int t, float& target) {
        uint8_t* x0img = slots + (size_t)(t - t0) * kSlotBytes;
        int64_t si = a.first + (int64_t)t * kTile + row;  // < 2 pool_n
        if (si >= a.pool_n) si -= a.pool_n;
        const float4 p = a.pool[si];
        target = p.w / a.out_scale;
        // core column cq + 4 ax of each axis: sin (cq < 2) or cos of
        // frequencies 8 (cq & 1) .. + 7
        const float c[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const float u = 2.f * (c[ax] - a.dom.lo[ax]) / (a.dom.hi[ax] - a.dom.lo[ax]) - 1.f;
            float f8[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float sv, cv;
                sincos_pi(a.ff.f[ax][8 * (cq & 1) + k] * u, sv, cv);
                f8[k] = cq < 2 ? sv : cv;
            }
            const uint4 u8 = pack8(f8);
            *reinterpret_cast<uint4*>(sXA + img_off(4 * ax + cq, row)) = u8;
            *reinterpret_cast<uint4*>(x0img + img_off(4 * ax + cq, row)) = u8;
        }
    };
    float target = 0.f;
    if (t0 < t1) features(t0, target);
    for (int t = t0; t < t1 && ok; t++) {
        uint8_t* x0img = slots + (size_t)(t - t0) * kSlotBytes;
        uint8_t* x1img = x0img + kX0Bytes;
        uint8_t* dz0img = x1img + kImgBytes;
        uint8_t* dz1img = dz0img + kImgBytes;
        // forward
        uint8_t* src = sXA;
        uint8_t* dst = sXB;
#pragma unroll 1
        for (int l = 0; l < kLayers && ok; l++) {
            to_tensor_core();
            if (threadIdx.x == 0) {
                tc_fence_after();
                const uint64_t ad = umma_desc(smem_u32(src), kCoreCol, 128);
                const uint64_t bd = umma_desc(w_addr + 2 * wb_off(l), kCoreCol, 128);
                if (l == 0) umma_chain<kIn / 16>(tmem + kTmWork, ad, 2 * kCoreCol, bd, 2 * kCoreCol, kIdescFwd, false);
                else umma_chain<kHidden / 16>(tmem + kTmWork, ad, 2 * kCoreCol, bd, 2 * kCoreCol, kIdescFwd, false);
                umma_commit(&bar);
            }
            float bv[32], w4c[32];
            load32(a.params + b_off(l) + 32 * cq, bv);
            if (l == kLayers - 1) load32(a.params + kHeadW + 32 * cq, w4c);
            ok = cta_wait(&bar, phase);
            if (!ok) break;
            float v[32];
            tmem_ld32(tmem + kTmWork + tl, v);
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                const float2 z = add2(make_float2(v[j], v[j + 1]), make_float2(bv[j], bv[j + 1]));
                v[j] = z.x;
                v[j + 1] = z.y;
            }
            if (l < kLayers - 1) {
#pragma unroll
                for (int g = 0; g < 4; g++)
                    *reinterpret_cast<uint4*>(zimg(l) + img_off(4 * cq + g, row)) = pack8(v + 8 * g);
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    const float2 z = make_float2(v[j], v[j + 1]);
                    const float2 x = mul2(z, sigmoid2(z));
                    v[j] = x.x;
                    v[j + 1] = x.y;
                }
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const uint4 u = pack8(v + 8 * g);
                    *reinterpret_cast<uint4*>(dst + img_off(4 * cq + g, row)) = u;
                    if (l == 0) *reinterpret_cast<uint4*>(x1img + img_off(4 * cq + g, row)) = u;
                }
                uint8_t* tmp = src;
                src = dst;
                dst = tmp;
            } else {
                // head: y from the BF16 activations, as in inference; the
                // four column quarters' sums meet in shared memory
                float2 y2 = v2(0.f);
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    const float2 z = make_float2(v[j], v[j + 1]);
                    const float2 sg = sigmoid2(z);
                    const float2 x = __bfloat1622float2(__float22bfloat162_rn(mul2(z, sg)));  // X4
                    const float2 w = make_float2(w4c[j], w4c[j + 1]);
                    y2 = fma2(x, w, y2);
                    const float2 d = mul2(w, silu_grad2(z, sg));  // dZ3 / dy = w4 silu'(z3)
                    w4c[j] = d.x;
                    w4c[j + 1] = d.y;
                    v[j] = x.x;
                    v[j + 1] = x.y;
                }
                ypart[cq][row] = y2.x + y2.y;
                __syncthreads();
                const float r = ((ypart[0][row] + ypart[1][row]) + (ypart[2][row] + ypart[3][row])) + b4 - target;
                const float dy = 2.f * r / (float)a.n;
                if (cq == 0) {
                    lsum = fmaf(r, r, lsum);
                    gb4 += dy;
                }
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    const float2 g = mul2(make_float2(v[j], v[j + 1]), v2(dy));         // w4's gradient terms
                    const float2 d = mul2(make_float2(w4c[j], w4c[j + 1]), v2(dy));     // dZ3
                    v[j] = g.x;
                    v[j + 1] = g.y;
                    w4c[j] = d.x;
                    w4c[j + 1] = d.y;
                }
#pragma unroll
                for (int g = 0; g < 4; g++)
                    *reinterpret_cast<uint4*>(sDZ + img_off(4 * cq + g, row)) = pack8(w4c + 8 * g);
                gw4 += warp_column_sums(v, lane);
            }
        }
        // backward: after the forward X2 is in XA and X3 in XB
#pragma unroll 1
        for (int l = kLayers - 1; l >= 1 && ok; l--) {
            to_tensor_core();
            if (threadIdx.x == 0) {
                tc_fence_after();
                if (l >= 2)
                    weight_grads(l == 3 ? kTmDW3 : kTmDW2, kTmDB + (l == 3 ? 16u : 0u), l == 3 ? xb_addr : xa_addr,
                                 kIdescDW, t > t0);
                // dX = dZ_l W_l: M = the tile's rows, N = 128 inputs, K = 128 outputs
                umma_chain<kHidden / 16>(tmem + kTmWork, umma_desc(dz_addr, kCoreCol, 128), 2 * kCoreCol,
                                         umma_desc(w_addr + 2 * wb_off(l), 128, kCoreCol), 256, kIdescDX, false);
                umma_commit(&bar);
            }
            // this thread's z_{l-1} (32 BF16 values) while the products run
            uint4 zr[4];
#pragma unroll
            for (int g = 0; g < 4; g++) zr[g] = *reinterpret_cast<const uint4*>(zimg(l - 1) + img_off(4 * cq + g, row));
            // and the next tile's features into XA (X2's products are done)
            if (l == 1 && t + 1 < t1) features(t + 1, target);
            ok = cta_wait(&bar, phase);
            if (!ok) break;
            float v[32], z[32];
            tmem_ld32(tmem + kTmWork + tl, v);
#pragma unroll
            for (int g = 0; g < 4; g++) unpack8(zr[g], z + 8 * g);
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                const float2 zz = make_float2(z[j], z[j + 1]);
                const float2 d = mul2(make_float2(v[j], v[j + 1]), silu_grad2(zz, sigmoid2(zz)));
                v[j] = d.x;
                v[j + 1] = d.y;
            }
#pragma unroll
            for (int g = 0; g < 4; g++) {
                const uint4 u = pack8(v + 8 * g);
                if (l > 1) *reinterpret_cast<uint4*>(sDZ + img_off(4 * cq + g, row)) = u;
                if (l == 2) *reinterpret_cast<uint4*>(dz1img + img_off(4 * cq + g, row)) = u;
                if (l == 1) *reinterpret_cast<uint4*>(dz0img + img_off(4 * cq + g, row)) = u;
            }
        }
    }
    float* part = a.partial + (size_t)blockIdx.x * kPartStride;
    const bool any = t1 > t0;
    // this thread's lane is output row `row` of each dW, its chunk the
    // columns 32 cq .. + 31 (layer 0 has three chunks); the bias sums are
    // column 0 of their 16-column blocks
    auto flush = [&](int l, uint32_t col0) {
        const int in = in_dim(l);
        if (32 * cq >= in) return;  // warp-uniform
        float v[32];
        if (any) tmem_ld32(tmem + col0 + tl, v);
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = any ? v[j] : 0.f;
        float4* d4 = reinterpret_cast<float4*>(part + w_off(l) + (size_t)row * in + 32 * cq);
#pragma unroll
        for (int j = 0; j < 8; j++) d4[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    };
    auto flush_bias = [&](int la, int lb) {  // db_la in column kTmDB, db_lb in kTmDB + 16
        if (cq != 0) return;
        float v[32];
        tmem_ld32(tmem + kTmDB + ((uint32_t)(32 * q) << 16), v);
        part[b_off(la) + row] = any ? v[0] : 0.f;
        part[b_off(lb) + row] = any ? v[16] : 0.f;
    };
    if (ok) {
        flush(2, kTmDW2);
        flush(3, kTmDW3);
        flush_bias(2, 3);
    }
    // dW_1, db_1, dW_0, db_0 over the CTA's tiles from the slots' images
    // (written by other threads of the CTA: the barrier orders their stores
    // before these reads, and the TMEM reads above before the MMAs below)
    tc_fence_before();
    __syncthreads();
    for (int t = t0; t < t1 && ok; t++) {
        const uint8_t* x0img = slots + (size_t)(t - t0) * kSlotBytes;
        const uint8_t* x1img = x0img + kX0Bytes;
        const uint8_t* dz0img = x1img + kImgBytes;
        const uint8_t* dz1img = dz0img + kImgBytes;
        for (int i = threadIdx.x; i < kImgBytes / 16; i += kTrainThreads) {
            cp_async16(sXA + 16 * i, x1img + 16 * i);
            cp_async16(sDZ + 16 * i, dz1img + 16 * i);
        }
        for (int i = threadIdx.x; i < kX0Bytes / 16; i += kTrainThreads) cp_async16(sXB + 16 * i, x0img + 16 * i);
        cp_async_wait_all();
        to_tensor_core();
        if (threadIdx.x == 0) {
            tc_fence_after();
            weight_grads(kTmDW2, kTmDB, xa_addr, kIdescDW, t > t0);
            umma_commit(&bar);
        }
        ok = cta_wait(&bar, phase);
        if (!ok) break;
        for (int i = threadIdx.x; i < kImgBytes / 16; i += kTrainThreads) cp_async16(sDZ + 16 * i, dz0img + 16 * i);
        cp_async_wait_all();
        to_tensor_core();
        if (threadIdx.x == 0) {
            tc_fence_after();
            weight_grads(kTmDW3, kTmDB + 16, xb_addr, kIdescDW0, t > t0);
            umma_commit(&bar);
        }
        ok = cta_wait(&bar, phase);
    }
    if (ok) {
        flush(1, kTmDW2);
        flush(0, kTmDW3);
        flush_bias(1, 0);
        // w4: column sums over the four lane quarters
        float* red = reinterpret_cast<float*>(sXA);  // [4][kHidden]
        red[q * kHidden + 32 * cq + lane] = gw4;
        // loss and b4 (rows are summed by the cq == 0 threads)
        float ls = lsum, gb = gb4;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            ls += __shfl_xor_sync(0xffffffffu, ls, o);
            gb += __shfl_xor_sync(0xffffffffu, gb, o);
        }
        if (cq == 0 && lane == 0) {
            ypart[0][q] = ls;
            ypart[1][q] = gb;
        }
        __syncthreads();
        if (threadIdx.x < kHidden) {
            const int c = threadIdx.x;
            part[kHeadW + c] = ((red[c] + red[kHidden + c]) + red[2 * kHidden + c]) + red[3 * kHidden + c];
        }
        if (threadIdx.x == 0) {
            part[kHeadB] = ((ypart[1][0] + ypart[1][1]) + ypart[1][2]) + ypart[1][3];
            part[kParams] = (((ypart[0][0] + ypart[0][1]) + ypart[0][2]) + ypart[0][3]) / (float)a.n;
        }
    } else {
        // as in k_mlp_infer: a second bounded wait for the pending commit
        // before the columns are freed; the status flag makes the host
        // discard the step's results either way
        if (threadIdx.x == 0) atomicExch(a.status, 1);
        uint32_t polls = 0;
        while (!mbar_try_wait(&bar, phase ^ 1u) && ++polls < 4 * kWaitLimit) {
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem_base, 512);
}

// The step's gradient: the sum of the CTAs' rows of `partial`, in CTA order.
// With lr > 0, Adam (beta 0.9 / 0.999, eps 1e-8) on the FP32 master weights
// and the BF16 copies refreshed; `grad` and `loss` receive the sums when not
// null.
__global__ void k_adam_partials(const float* partial, int parts, float* p, float* m, float* v, float lr, float c1,
                                float c2, __nv_bfloat16* wb, LayerMap lm, float* grad, float* loss) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= kParams; i += gridDim.x * blockDim.x) {
        float gi = 0.f;
        for (int c = 0; c < parts; c++) gi += partial[(size_t)c * kPartStride + i];
        if (i == kParams) {  // the loss
            if (loss) *loss = gi;
            continue;
        }
        if (grad) grad[i] = gi;
        if (!(lr > 0.f)) continue;
        const float mi = 0.9f * m[i] + 0.1f * gi;
        const float vi = 0.999f * v[i] + 0.001f * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
        p[i] = pi;
#pragma unroll
        for (int l = 0; l < kLayers; l++) {
            const int rel = i - lm.w[l];
            if (rel >= 0 && rel < kHidden * lm.in[l]) wb[lm.wb[l] + rel] = __float2bfloat16_rn(pi);
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 density: the 2D fBm heightfield (+ 3D fBm caves) in double precision,
// with the exact simplex constants, over the same permutation image and
// gradient table, as the reference the surrogate's and the FP32 density's
// errors are measured against.
// ---------------------------------------------------------------------------

__device__ double snoise2_f64(const uint8_t* perm, const float* grad, double px, double py) {
    const double F2 = 0.36602540378443864676, G2 = 0.21132486540518711775;
    const double s = (px + py) * F2;
    const double fi = floor(px + s), fj = floor(py + s);
    const double t = (fi + fj) * G2;
    const double x0 = px - (fi - t), y0 = py - (fj - t);
    const int i = (int)fi, j = (int)fj;
    const int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    const double xs[3] = {x0, x0 - i1 + G2, x0 - 1.0 + 2.0 * G2};
    const double ys[3] = {y0, y0 - j1 + G2, y0 - 1.0 + 2.0 * G2};
    const int oi[3] = {0, i1, 1}, oj[3] = {0, j1, 1};
    double n = 0.0;
    for (int c = 0; c < 3; c++) {
        double tt = 0.5 - xs[c] * xs[c] - ys[c] * ys[c];
        if (tt <= 0.0) continue;
        const int k = perm[texel(j + oj[c], i + oi[c])] & 15;
        tt *= tt;
        n += tt * tt * ((double)grad[4 * k] * xs[c] + (double)grad[4 * k + 1] * ys[c]);
    }
    return 70.0 * n;
}

__device__ double snoise3_f64(const uint8_t* perm, const float* grad, double px, double py, double pz) {
    const double F3 = 1.0 / 3.0, G3 = 1.0 / 6.0;
    const double s = (px + py + pz) * F3;
    const double fi = floor(px + s), fj = floor(py + s), fk = floor(pz + s);
    const double t = (fi + fj + fk) * G3;
    const double x0 = px - (fi - t), y0 = py - (fj - t), z0 = pz - (fk - t);
    const int i = (int)fi, j = (int)fj, k = (int)fk;
    // the reference's ranking (simplex.cl:133-156)
    const int sxy = x0 >= y0, sxz = x0 >= z0, syz = y0 >= z0;
    const int rx = sxy + sxz, ry = (1 - sxy) + syz, rz = (1 - sxz) + (1 - syz);
    const int o2[3] = {rx >= 1, ry >= 1, rz >= 1}, o1[3] = {rx >= 2, ry >= 2, rz >= 2};
    const int oi[4] = {0, o1[0], o2[0], 1}, oj[4] = {0, o1[1], o2[1], 1}, ok[4] = {0, o1[2], o2[2], 1};
    double n = 0.0;
    for (int c = 0; c < 4; c++) {
        const double x = x0 - oi[c] + c * G3, y = y0 - oj[c] + c * G3, z = z0 - ok[c] + c * G3;
        double tt = 0.6 - x * x - y * y - z * z;
        if (tt <= 0.0) continue;
        const int a = perm[texel(j + oj[c], i + oi[c])];
        const int g = perm[texel(k + ok[c], alpha_column(a))] & 15;
        tt *= tt;
        n += tt * tt * ((double)grad[4 * g] * x + (double)grad[4 * g + 1] * y + (double)grad[4 * g + 2] * z);
    }
    return 32.0 * n;
}

__global__ void k_density_f64(const float4* pts, int64_t n, const uint8_t* perm, const float* grad, DensityParams d,
                              double* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 p = pts[i];
        double fx = p.x * (double)d.freq2, fz = p.z * (double)d.freq2, amp = 1.0, h = 0.0;
        for (int o = 0; o < d.octaves2; o++) {
            h += snoise2_f64(perm, grad, fx, fz) * amp;
            fx *= d.lacunarity2;
            fz *= d.lacunarity2;
            amp *= d.gain2;
        }
        double v = (double)p.y - (double)d.amp2 * h;
        if (d.mode == LVN_DENSITY_CAVES) {
            double gx = p.x * (double)d.freq3, gy = p.y * (double)d.freq3, gz = p.z * (double)d.freq3, a3 = 1.0,
                   c = 0.0;
            for (int o = 0; o < d.octaves3; o++) {
                c += snoise3_f64(perm, grad, gx, gy, gz) * a3;
                gx *= d.lacunarity3;
                gy *= d.lacunarity3;
                gz *= d.lacunarity3;
                a3 *= d.gain3;
            }
            v += (double)d.amp3 * c;
        }
        out[i] = v;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define SG_CK(x)                                       \
    do {                                               \
        const cudaError_t e__ = (x);                   \
        if (e__ != cudaSuccess) {                      \
            cudaGetLastError();                        \
            return e__ == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA; \
        }                                              \
    } while (0)

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t b) {
        if (b <= bytes) return LVN_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        SG_CK(cudaMalloc(&p, b));
        bytes = b;
        return LVN_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

LayerMap layer_map() {
    LayerMap lm;
    for (int l = 0; l < kLayers; l++) {
        lm.w[l] = w_off(l);
        lm.b[l] = b_off(l);
        lm.in[l] = kIn_[l];
        lm.wb[l] = wb_off(l);
    }
    return lm;
}

}  // namespace
}  // namespace lvn

using namespace lvn;

struct lvn_surrogate {
    Domain dom;
    FeatureFreqs ff;
    float out_scale = 8.f;  // the network predicts density / out_scale
    cudaStream_t stream = nullptr;
    Buf params, grads, adam_m, adam_v, wb, loss, status;
    Buf loss_hist;  // one loss per training step, read back once per lvn_surrogate_train
    // points and densities of host calls
    int cap = 0;
    Buf pts, dens;
    Buf pool;  // training samples
    int num_sms = 0;

    // fused inference of n points (explicit `pts`, or `lattices` of dim^3) into out (device)
    int infer(const float4* pts_d, const float4* lattices_d, int dim, int64_t n, float* out_d) {
        static bool configured = false;
        if (!configured) {
            SG_CK(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem));
            configured = true;
        }
        InferArgs a;
        std::memset(&a, 0, sizeof(a));
        a.pts = pts_d;
        a.lattices = lattices_d;
        a.dim = dim;
        a.n = n;
        a.wb = wb.as<__nv_bfloat16>();
        a.params = params.as<float>();
        a.dom = dom;
        a.ff = ff;
        a.out_scale = out_scale;
        a.out = out_d;
        a.status = status.as<int>();
        const int64_t tiles = (n + kTile - 1) / kTile;
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(num_sms, (tiles + kInferWG - 1) / kInferWG));
        k_mlp_infer<<<grid, 128 * kInferWG, kInferSmem, stream>>>(a);
        SG_CK(cudaGetLastError());
        return LVN_OK;
    }
    int64_t pool_n = 0;
    int64_t pool_next = 0;
    int step = 0;
    Buf train_scratch, partial;  // k_mlp_train's per-CTA images and gradient rows

    // one fused forward + backward over rows first .. first + n - 1 (mod
    // pool_n) of pool_d; *parts = the rows of `partial` it writes
    int train_launch(const float4* pool_d, int64_t pool_n_, int64_t first, int n, int* parts) {
        static bool configured = false;
        if (!configured) {
            SG_CK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem));
            configured = true;
        }
        const int ntiles = n / kTile;
        const int tpc = (ntiles + num_sms - 1) / num_sms;
        const int grid = (ntiles + tpc - 1) / tpc;
        int rc;
        if ((rc = train_scratch.ensure((size_t)grid * ((size_t)tpc * kSlotBytes + kTransientBytes)))) return rc;
        if ((rc = partial.ensure(sizeof(float) * (size_t)grid * kPartStride))) return rc;
        TrainArgs a;
        std::memset(&a, 0, sizeof(a));
        a.pool = pool_d;
        a.pool_n = pool_n_;
        a.first = first;
        a.n = n;
        a.tiles_per_cta = tpc;
        a.wb = wb.as<__nv_bfloat16>();
        a.params = params.as<float>();
        a.dom = dom;
        a.ff = ff;
        a.out_scale = out_scale;
        a.scratch = train_scratch.as<uint8_t>();
        a.partial = partial.as<float>();
        a.status = status.as<int>();
        k_mlp_train<<<grid, kTrainThreads, kTrainSmem, stream>>>(a);
        SG_CK(cudaGetLastError());
        *parts = grid;
        return LVN_OK;
    }

    int ensure_batch(int n) {
        if (n <= cap) return LVN_OK;
        int rc;
        if ((rc = pts.ensure(sizeof(float4) * n))) return rc;
        if ((rc = dens.ensure(4ull * n))) return rc;
        cap = n;
        return LVN_OK;
    }
};

namespace {

int check_status(lvn_surrogate* s) {
    int st = 0;
    SG_CK(cudaMemcpyAsync(&st, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SG_CK(cudaStreamSynchronize(s->stream));
    return st ? LVN_ERR_DEVICE_STATUS : LVN_OK;
}

int upload_samples(lvn_surrogate* s, const float* host, int n) {
    int rc = s->ensure_batch(n);
    if (rc) return rc;
    SG_CK(cudaMemcpyAsync(s->pts.p, host, sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream));
    return LVN_OK;
}

}  // namespace

extern "C" {

lvn_surrogate* lvn_surrogate_create(const float domain_min[3], const float domain_max[3], uint64_t seed) {
    if (!domain_min || !domain_max) return nullptr;
    for (int a = 0; a < 3; a++)
        if (!(domain_max[a] > domain_min[a])) return nullptr;
    lvn_surrogate* s = new lvn_surrogate();
    for (int a = 0; a < 3; a++) {
        s->dom.lo[a] = domain_min[a];
        s->dom.hi[a] = domain_max[a];
        // frequencies from one period over the domain to a 2-voxel period
        const double top = std::log2(std::max(2.0, (double)(domain_max[a] - domain_min[a]) / 2.0));
        for (int k = 0; k < kFreqs; k++) s->ff.f[a][k] = (float)std::exp2(top * k / (kFreqs - 1));
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev);
    bool ok = !s->params.ensure(4ull * kParams) && !s->grads.ensure(4ull * kParams) && !s->adam_m.ensure(4ull * kParams) &&
              !s->adam_v.ensure(4ull * kParams) && !s->wb.ensure(2ull * kWb) &&
              !s->loss.ensure(4) && !s->status.ensure(4);
    // PyTorch's Linear initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in)), from splitmix64(seed)
    std::vector<float> h(kParams);
    uint64_t st = seed;
    auto next = [&st]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t x = st;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (float)(x >> 40) * (1.f / 16777216.f);
    };
    for (int l = 0; l <= kLayers; l++) {
        const int fan_in = l < kLayers ? kIn_[l] : kHidden;
        const int wo = l < kLayers ? w_off(l) : kHeadW, bo = l < kLayers ? b_off(l) : kHeadB;
        const int nw = l < kLayers ? kHidden * fan_in : kHidden, nb = l < kLayers ? kHidden : 1;
        const float bound = 1.f / std::sqrt((float)fan_in);
        for (int i = 0; i < nw; i++) h[wo + i] = (2.f * next() - 1.f) * bound;
        for (int i = 0; i < nb; i++) h[bo + i] = (2.f * next() - 1.f) * bound;
    }
    if (ok && lvn_surrogate_set_params(s, h.data(), kParams) != LVN_OK) ok = false;
    if (!ok) {
        lvn_surrogate_destroy(s);
        return nullptr;
    }
    return s;
}

void lvn_surrogate_destroy(lvn_surrogate* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    Buf* bufs[] = {&s->params, &s->grads, &s->adam_m, &s->adam_v, &s->wb,   &s->loss,          &s->status,
                   &s->pts,    &s->dens,  &s->pool,   &s->loss_hist, &s->train_scratch, &s->partial};
    for (Buf* b : bufs) b->release();
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int32_t lvn_surrogate_num_params(void) { return kParams; }

int lvn_surrogate_set_params(lvn_surrogate* s, const float* host, int64_t n) {
    if (!s || !host || n != kParams) return LVN_ERR_INVALID;
    SG_CK(cudaMemcpyAsync(s->params.p, host, 4ull * kParams, cudaMemcpyHostToDevice, s->stream));
    SG_CK(cudaMemsetAsync(s->adam_m.p, 0, 4ull * kParams, s->stream));
    SG_CK(cudaMemsetAsync(s->adam_v.p, 0, 4ull * kParams, s->stream));
    SG_CK(cudaMemsetAsync(s->status.p, 0, 4, s->stream));
    k_to_bf16<<<64, 256, 0, s->stream>>>(s->params.as<float>(), kParams, s->wb.as<__nv_bfloat16>(), layer_map());
    SG_CK(cudaGetLastError());
    s->step = 0;
    SG_CK(cudaStreamSynchronize(s->stream));
    return LVN_OK;
}

int lvn_surrogate_get_params(lvn_surrogate* s, float* host, int64_t n) {
    if (!s || !host || n < kParams) return LVN_ERR_INVALID;
    SG_CK(cudaMemcpyAsync(host, s->params.p, 4ull * kParams, cudaMemcpyDeviceToHost, s->stream));
    SG_CK(cudaStreamSynchronize(s->stream));
    return kParams;
}

int lvn_surrogate_sample(lvn_surrogate* s, int64_t n, uint64_t seed, float* host_out) {
    if (!s || n <= 0) return LVN_ERR_INVALID;
    const GlobalView gv = global_view();
    if (!gv.initialised) return LVN_ERR_NOT_INITIALISED;
    int rc = s->pool.ensure(sizeof(float4) * (size_t)n);
    if (rc) return rc;
    float band = 0.f, rem[kCaveSteps + 1];
    int32_t dom_by_solid[9];
    density_fields(gv.density, gv.default_material, &band, rem, dom_by_solid);
    k_samples<<<gv.num_sms * 8, 256, 0, s->stream>>>(s->pool.as<float4>(), (int)n, seed, s->dom, gv.perm_t3,
                                                     gv.grad, gv.density, band);
    SG_CK(cudaGetLastError());
    s->pool_n = n;
    s->pool_next = 0;
    if (host_out) SG_CK(cudaMemcpyAsync(host_out, s->pool.p, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    SG_CK(cudaStreamSynchronize(s->stream));
    return LVN_OK;
}

int lvn_surrogate_grad(lvn_surrogate* s, const float* samples, int32_t n, float* grad_out, float* loss_out) {
    if (!s || !samples || n <= 0 || n % kTile) return LVN_ERR_INVALID;
    int rc = upload_samples(s, samples, n);
    if (rc) return rc;
    int parts = 0;
    if ((rc = s->train_launch(s->pts.as<float4>(), n, 0, n, &parts))) return rc;
    k_adam_partials<<<(kParams + 256) / 256, 256, 0, s->stream>>>(s->partial.as<float>(), parts, nullptr, nullptr,
                                                                   nullptr, 0.f, 0.f, 0.f, nullptr, layer_map(),
                                                                   s->grads.as<float>(), s->loss.as<float>());
    SG_CK(cudaGetLastError());
    if ((rc = check_status(s))) return rc;
    if (grad_out) SG_CK(cudaMemcpy(grad_out, s->grads.p, 4ull * kParams, cudaMemcpyDeviceToHost));
    if (loss_out) SG_CK(cudaMemcpy(loss_out, s->loss.p, 4, cudaMemcpyDeviceToHost));
    return LVN_OK;
}

int lvn_surrogate_train(lvn_surrogate* s, int32_t steps, int32_t batch, float lr, float* losses) {
    if (!s || steps < 0 || batch <= 0 || batch % kTile || !(lr > 0.f)) return LVN_ERR_INVALID;
    if (s->pool_n < batch) return LVN_ERR_INVALID;  // lvn_surrogate_sample first
    int rc;
    const LayerMap lm = layer_map();
    // the losses stay on the device until the end, so the host never waits
    // on a step and the launches queue ahead of the GPU
    if (steps > 0 && (rc = s->loss_hist.ensure(sizeof(float) * (size_t)steps))) return rc;
    for (int it = 0; it < steps; it++) {
        // the next `batch` samples of the pool (wrapping), read in place
        const int64_t first = s->pool_next;
        s->pool_next = (first + batch) % s->pool_n;
        int parts = 0;
        if ((rc = s->train_launch(s->pool.as<float4>(), s->pool_n, first, batch, &parts))) return rc;
        s->step++;
        const float c1 = 1.f / (1.f - std::pow(0.9f, (float)s->step));
        const float c2 = 1.f / (1.f - std::pow(0.999f, (float)s->step));
        k_adam_partials<<<(kParams + 256) / 256, 256, 0, s->stream>>>(
            s->partial.as<float>(), parts, s->params.as<float>(), s->adam_m.as<float>(), s->adam_v.as<float>(), lr, c1,
            c2, s->wb.as<__nv_bfloat16>(), lm, nullptr, s->loss_hist.as<float>() + it);
        SG_CK(cudaGetLastError());
    }
    if (losses && steps > 0)
        SG_CK(cudaMemcpyAsync(losses, s->loss_hist.p, sizeof(float) * (size_t)steps, cudaMemcpyDeviceToHost, s->stream));
    return check_status(s);
}

int lvn_surrogate_eval(lvn_surrogate* s, const float* points, int64_t n, float* density, int32_t memory) {
    if (!s || !points || !density || n <= 0) return LVN_ERR_INVALID;
    int rc;
    if (memory == LVN_MEMORY_DEVICE) {
        if ((rc = s->infer(reinterpret_cast<const float4*>(points), nullptr, 0, n, density))) return rc;
        return check_status(s);
    }
    // host arrays: staged through the batch buffers, 2^20 points at a time
    const int64_t chunk = 1 << 20;
    if ((rc = s->ensure_batch((int)std::min<int64_t>(chunk, (n + kTile - 1) / kTile * kTile)))) return rc;
    for (int64_t first = 0; first < n; first += chunk) {
        const int m = (int)std::min<int64_t>(chunk, n - first);
        SG_CK(cudaMemcpyAsync(s->pts.p, points + 4 * first, sizeof(float4) * m, cudaMemcpyHostToDevice, s->stream));
        if ((rc = s->infer(s->pts.as<float4>(), nullptr, 0, m, s->dens.as<float>()))) return rc;
        SG_CK(cudaMemcpyAsync(density + first, s->dens.p, sizeof(float) * m, cudaMemcpyDeviceToHost, s->stream));
    }
    return check_status(s);
}

int lvn_surrogate_eval_lattices(lvn_surrogate* s, const float* lattices, int32_t count, int32_t dim, float* density) {
    if (!s || !lattices || !density || count < 0 || dim <= 0) return LVN_ERR_INVALID;
    const int64_t n = (int64_t)count * dim * dim * dim;
    if (n == 0) return LVN_OK;
    const int rc = s->infer(nullptr, reinterpret_cast<const float4*>(lattices), dim, n, density);
    if (rc) return rc;
    return check_status(s);
}

int lvn_surrogate_domain(const lvn_surrogate* s, float domain_min[3], float domain_max[3]) {
    if (!s || !domain_min || !domain_max) return LVN_ERR_INVALID;
    for (int a = 0; a < 3; a++) {
        domain_min[a] = s->dom.lo[a];
        domain_max[a] = s->dom.hi[a];
    }
    return LVN_OK;
}

void* lvn_surrogate_get_stream(lvn_surrogate* s) { return s ? (void*)s->stream : nullptr; }

int lvn_density_f64(const float* points, int64_t n, double* density) {
    if (!points || !density || n <= 0) return LVN_ERR_INVALID;
    const GlobalView gv = global_view();
    if (!gv.initialised) return LVN_ERR_NOT_INITIALISED;
    if (gv.density.mode != LVN_DENSITY_FBM2D && gv.density.mode != LVN_DENSITY_CAVES) return LVN_ERR_INVALID;
    Buf p, o;
    int rc;
    if ((rc = p.ensure(sizeof(float4) * (size_t)n)) || (rc = o.ensure(sizeof(double) * (size_t)n))) {
        p.release();
        return rc;
    }
    cudaMemcpy(p.p, points, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice);
    k_density_f64<<<gv.num_sms * 4, 256>>>(p.as<float4>(), n, gv.perm, gv.grad, gv.density, o.as<double>());
    const cudaError_t e = cudaGetLastError();
    const cudaError_t c = cudaMemcpy(density, o.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    p.release();
    o.release();
    return e == cudaSuccess && c == cudaSuccess ? LVN_OK : LVN_ERR_CUDA;
}

}  // extern "C"
