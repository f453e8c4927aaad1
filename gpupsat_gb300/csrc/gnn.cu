// Learned seeding: the kernels of a 3-layer, 64-wide message-passing network
// over the variable-clause graph of a batch of formulas (bf16 storage, fp32
// accumulation), forward and backward, and its optimiser step.
//
// The network (no counterpart in the reference; it seeds the reference's
// DecisionStrategy/VSIDS activities and phases, and the JobChooser's split
// variables):
//   H_v^0 = relu(F_v Win + bin), H_c^0 = hc0        (F_v: variable features)
//   [A+ | A- | Zv] = H_v^{l-1} [W+ | W- | Wv] + [0 | 0 | bv]
//   H_c^l = relu( sum over the literals (v, s) of c of A_s[v] + H_c^{l-1} Wc + bc )
//   [B+ | B-] = H_c^l [U+ | U-]
//   H_v^l = relu( sum over the clauses (c, s) holding v of B_s[c] + Zv )
//   score_v = H_v^3 . ws + bs,  phase_v = H_v^3 . wp + bp
//
// Kernels:
//   mm_kernel       Y = X B^T + bias, rows x K times K x N (K, N multiples of 64,
//                   K <= 192, N <= 256).  Tiles of 128 rows: TMA loads the X tile
//                   and B into shared memory, one thread issues tcgen05.mma
//                   (kind::f16, bf16 in, fp32 accumulator in tensor memory,
//                   M = 128, N, K = 16 per instruction), the four warps read the
//                   accumulator back with tcgen05.ld and store bf16 rows.
//                   Every linear map of the forward pass and every data
//                   gradient of the backward pass is one call.
//   wgrad_kernel    dW += X^T dY (weight gradients; K = rows is the long axis):
//                   rows transposed into shared memory in register 8 x 8 blocks,
//                   tcgen05.mma (M = 128 with X^T zero-padded, N, K = 16) into a
//                   tensor-memory accumulator per block, double-buffered staging
//   gather_kernel   out[s] = act( scale[s] * sum_e src_{sign e}[idx e] + Z[s] )
//                   (message means: scale = 1 / degree)
//   gather_split_kernel  outP[s], outN[s] = sums of scale[idx e] * src[idx e] over
//                   the positive / negative edges of s   (backward of a message mean)
//   relu_bwd, colsum, broadcast, head_loss, adam, pack: elementwise pieces.
//
// Shared-memory operand layout for tcgen05 (no swizzle, K-major): an operand of
// R rows x K bf16 is stored as K/8 slabs; slab j holds elements [8j, 8j+8) of
// every row, rows 16 bytes apart, so a core matrix (8 rows x 16 bytes) is 128
// contiguous bytes, the next 8 rows start 128 bytes later (stride byte offset)
// and the next 8 elements of K start R*16 bytes later (leading byte offset).
// One TMA box {8 elements, R rows} fills one slab.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "internal.h"

namespace gpsat {
namespace gnn {

constexpr int TILE = 128;          // rows per tile = tensor-memory lanes
constexpr int MAXK = 192;
constexpr int MAXN = 256;
constexpr long long WAIT_LIMIT = 1ll << 26;   // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait on phase `parity`; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (long long i = 0; i < WAIT_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: kind::f16, bf16 A and B (both K-major), fp32 D
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

struct MmArgs {
    int rows, K, N;
    int relu;                // epilogue: max(0, .)
    const float *bias;       // N floats or null
    __nv_bfloat16 *Y;        // rows x ldy
    int ldy;
    int *err;                // set to 1 when a wait gave up
};

// One 128-row tile per block, 128 threads.  Dynamic shared memory:
// [X tile 128*K*2][B N*K*2][2 mbarriers][tensor-memory address]
__global__ void __launch_bounds__(128) mm_kernel(const __grid_constant__ CUtensorMap xmap,
                                                 const __grid_constant__ CUtensorMap bmap, MmArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int K = a.K, N = a.N;
    unsigned char *xs = sm;
    unsigned char *bs = sm + TILE * K * 2;
    uint64_t *bars = reinterpret_cast<uint64_t *>(bs + N * K * 2);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * TILE;
    // tensor-memory columns: a power of two >= 32 covering N
    const uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    bool ok = true;
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)(TILE * K * 2 + N * K * 2);
        mbar_expect_tx(&bars[0], bytes);
        for (int j = 0; j < K / 8; j++) {
            tma_load_2d(xs + j * TILE * 16, &xmap, 8 * j, row0, &bars[0]);
            tma_load_2d(bs + j * N * 16, &bmap, 8 * j, 0, &bars[0]);
        }
        ok = mbar_wait(&bars[0], 0);
        if (ok) {
            const uint32_t idesc = instr_desc(TILE, N);
            const uint32_t xa = smem_u32(xs), ba = smem_u32(bs);
            // one instruction per 16 elements of K = two slabs
            for (int k = 0; k < K / 16; k++) {
                const uint64_t ad = smem_desc(xa + 2 * k * TILE * 16, TILE * 16, 128);
                const uint64_t bd = smem_desc(ba + 2 * k * N * 16, N * 16, 128);
                const uint32_t acc = k > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bars[1]))
                         : "memory");
        }
    }
    ok = __syncthreads_and(ok);
    if (ok) ok = mbar_wait(&bars[1], 0);
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (ok) {
        // warp w reads tensor-memory lanes [32w, 32w + 32): row 32w + lane
        const int r = row0 + warp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                "[%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(lane_base + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < a.rows) {
                uint32_t packed[16];
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    float x0 = __uint_as_float(v[2 * i]), x1 = __uint_as_float(v[2 * i + 1]);
                    if (a.bias) {
                        x0 += a.bias[c0 + 2 * i];
                        x1 += a.bias[c0 + 2 * i + 1];
                    }
                    if (a.relu) {
                        x0 = fmaxf(x0, 0.f);
                        x1 = fmaxf(x1, 0.f);
                    }
                    __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
                    packed[i] = *reinterpret_cast<uint32_t *>(&h);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(a.Y + (size_t)r * a.ldy + c0);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(a.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------- weight gradients
// dW[64 x N] += X[rows x 64]^T dY[rows x N] on the tensor cores.  The long
// axis (rows) is the contraction axis: a block takes chunks of WT_R rows
// (strided over the grid) and, per chunk, its 128 threads transpose the rows
// of X and dY in registers (8 x 8 bf16 blocks) into the no-swizzle K-major
// operand layout above -- A = X^T as 128 rows (channels; rows 64..127 stay
// zero), B = dY^T as N rows, K = the chunk's rows -- make the generic-proxy
// writes visible to the tensor core (fence.proxy.async), and one thread
// issues WT_R / 16 tcgen05.mma (M = 128, N, K = 16) accumulating into one fp32
// matrix in tensor memory for all of the block's chunks.  Staging is double
// buffered: the block fills one buffer while the tensor core reads the
// other.  At the end warps 0-1 read lanes 0..63 back and add them into dW
// (one atomic per output per block).
constexpr int WT_R = 128;
constexpr int WT_MAXN = 192;

__device__ __forceinline__ void transpose8x8(const uint4 in[8], uint4 out[8])
{
    // in[r] = row r (8 bf16: channels 0..7); out[c] = channel c (8 bf16: rows 0..7)
    const uint32_t *w = reinterpret_cast<const uint32_t *>(in);   // w[4 r + c / 2]
    uint32_t *o = reinterpret_cast<uint32_t *>(out);
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
        for (int q = 0; q < 4; q++)
            o[4 * c + q] = __byte_perm(w[4 * (2 * q) + (c >> 1)], w[4 * (2 * q + 1) + (c >> 1)],
                                       (c & 1) ? 0x7632 : 0x5410);
}

struct WgArgs {
    const __nv_bfloat16 *X;
    int ldx;
    const __nv_bfloat16 *dY;
    int ldy;
    int rows, N;
    float *dW;
    int *err;
};

// Dynamic shared memory: [A 2 x 128*WT_R*2][B 2 x N*WT_R*2][2 mbarriers][tensor-memory address]
__global__ void __launch_bounds__(128) wgrad_kernel(WgArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int N = a.N;
    constexpr int ABYTES = 128 * WT_R * 2;
    const int BBYTES = N * WT_R * 2;
    unsigned char *As = sm;
    unsigned char *Bs = sm + 2 * ABYTES;
    uint64_t *bars = reinterpret_cast<uint64_t *>(Bs + 2 * BBYTES);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = N <= 64 ? 64 : N <= 128 ? 128 : 256;
    const int nchunks = (a.rows + WT_R - 1) / WT_R;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the padding rows 64..127 of both A buffers are zero for good
    for (int i = tid; i < 2 * ABYTES / 16; i += 128) {
        const int buf = i / (ABYTES / 16), w = i % (ABYTES / 16);
        const int row = (w % (128 * 16 / 16));   // 16-byte row inside its slab
        if (row >= 64) reinterpret_cast<uint4 *>(As + buf * ABYTES)[w] = make_uint4(0, 0, 0, 0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t idesc = instr_desc(128, N);

    bool ok = true;
    int issued = 0;                       // chunks multiplied by this block
    uint32_t phase[2] = {0u, 0u};         // parity of each buffer's next completion
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int buf = issued & 1;
        // the tensor core has finished reading this buffer (two chunks ago)
        if (issued >= 2) {
            bool w = true;
            if (tid == 0) w = mbar_wait(&bars[buf], phase[buf]);
            ok = __syncthreads_and(ok && w);
            phase[buf] ^= 1u;
            if (!ok) break;
        }
        unsigned char *A = As + buf * ABYTES;
        unsigned char *B = Bs + buf * BBYTES;
        const int r0 = ch * WT_R;
        // 8 x 8 blocks: X has (WT_R / 8) x 8 of them, dY (WT_R / 8) x (N / 8)
        const int nbx = (WT_R / 8) * 8, nby = (WT_R / 8) * (N / 8);
        for (int bkt = tid; bkt < nbx + nby; bkt += 128) {
            const bool isx = bkt < nbx;
            const int b = isx ? bkt : bkt - nbx;
            const int cols = isx ? 8 : N / 8;
            const int rb = b / cols, cb = b % cols;
            const __nv_bfloat16 *src = isx ? a.X : a.dY;
            const int ld = isx ? a.ldx : a.ldy;
            uint4 in[8], out[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const int row = r0 + 8 * rb + r;
                in[r] = row < a.rows ? *reinterpret_cast<const uint4 *>(src + (size_t)row * ld + 8 * cb)
                                     : make_uint4(0, 0, 0, 0);
            }
            transpose8x8(in, out);
            // operand row (channel) 8 cb + c, K elements [8 rb, 8 rb + 8): slab rb
            unsigned char *dst = isx ? A + rb * (128 * 16) : B + rb * (N * 16);
#pragma unroll
            for (int c = 0; c < 8; c++) *reinterpret_cast<uint4 *>(dst + (8 * cb + c) * 16) = out[c];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t aa = smem_u32(A), ba = smem_u32(B);
            for (int k = 0; k < WT_R / 16; k++) {
                const uint64_t ad = smem_desc(aa + 2 * k * 128 * 16, 128 * 16, 128);
                const uint64_t bd = smem_desc(ba + 2 * k * N * 16, N * 16, 128);
                const uint32_t acc = (issued > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bars[buf]))
                         : "memory");
        }
        issued++;
    }
    // wait for the products still in flight (the last one or two buffers)
    for (int k = issued >= 2 ? issued - 2 : 0; k < issued && ok; k++) {
        const int buf = k & 1;
        bool w = true;
        if (tid == 0) w = mbar_wait(&bars[buf], phase[buf]);
        ok = __syncthreads_and(ok && w);
        phase[buf] ^= 1u;
    }
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && issued > 0 && warp < 2) {
        // warp w reads tensor-memory lanes [32w, 32w + 32): dW row 32w + lane
        const int i = warp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                "[%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(lane_base + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 32; q++) atomicAdd(&a.dW[(size_t)i * N + c0 + q], __uint_as_float(v[q]));
        }
    } else if (!ok && tid == 0 && a.err) {
        atomicExch(a.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------- message sums
// One warp per segment; lane l holds channels 2l, 2l+1.  An edge is
// (row << 1) | positive.
__global__ void gather_kernel(const int64_t *seg_off, const int32_t *edges, int segs, const __nv_bfloat16 *srcP,
                              const __nv_bfloat16 *srcN, int lds, const float *seg_scale, const __nv_bfloat16 *Z,
                              int ldz, __nv_bfloat16 *out, int ldo, int relu)
{
    const int lane = threadIdx.x & 31;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < segs; s += (gridDim.x * blockDim.x) >> 5) {
        float2 acc = make_float2(0.f, 0.f);
        const int64_t e0 = seg_off[s], e1 = seg_off[s + 1];
        for (int64_t e = e0; e < e1; e++) {
            const int32_t ed = edges[e];
            const __nv_bfloat16 *src = (ed & 1) ? srcP : srcN;
            const float2 f =
                __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(src + (size_t)(ed >> 1) * lds + 2 * lane));
            acc.x += f.x;
            acc.y += f.y;
        }
        if (seg_scale) {
            const float sc = seg_scale[s];
            acc.x *= sc;
            acc.y *= sc;
        }
        if (Z) {
            const float2 z = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(Z + (size_t)s * ldz + 2 * lane));
            acc.x += z.x;
            acc.y += z.y;
        }
        if (relu) {
            acc.x = fmaxf(acc.x, 0.f);
            acc.y = fmaxf(acc.y, 0.f);
        }
        *reinterpret_cast<__nv_bfloat162 *>(out + (size_t)s * ldo + 2 * lane) = __floats2bfloat162_rn(acc.x, acc.y);
    }
}

__global__ void gather_split_kernel(const int64_t *seg_off, const int32_t *edges, int segs,
                                    const __nv_bfloat16 *src, int lds, const float *src_scale, __nv_bfloat16 *outP,
                                    __nv_bfloat16 *outN, int ldo)
{
    const int lane = threadIdx.x & 31;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < segs; s += (gridDim.x * blockDim.x) >> 5) {
        float2 p = make_float2(0.f, 0.f), n = make_float2(0.f, 0.f);
        const int64_t e0 = seg_off[s], e1 = seg_off[s + 1];
        for (int64_t e = e0; e < e1; e++) {
            const int32_t ed = edges[e];
            float2 f =
                __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(src + (size_t)(ed >> 1) * lds + 2 * lane));
            if (src_scale) {
                const float sc = src_scale[ed >> 1];
                f.x *= sc;
                f.y *= sc;
            }
            if (ed & 1) {
                p.x += f.x;
                p.y += f.y;
            } else {
                n.x += f.x;
                n.y += f.y;
            }
        }
        *reinterpret_cast<__nv_bfloat162 *>(outP + (size_t)s * ldo + 2 * lane) = __floats2bfloat162_rn(p.x, p.y);
        *reinterpret_cast<__nv_bfloat162 *>(outN + (size_t)s * ldo + 2 * lane) = __floats2bfloat162_rn(n.x, n.y);
    }
}

// dpre = dout where h > 0 (h = relu(pre), so h > 0 exactly where pre > 0)
__global__ void relu_bwd_kernel(const __nv_bfloat16 *dout, int ldd, const __nv_bfloat16 *h, int ldh, int rows,
                                __nv_bfloat16 *dpre, int ldp)
{
    const int64_t total = (int64_t)rows * 32;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t >> 5;
        const int c = 2 * (int)(t & 31);
        const float2 g = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(dout + r * ldd + c));
        const float2 x = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(h + r * ldh + c));
        *reinterpret_cast<__nv_bfloat162 *>(dpre + r * ldp + c) =
            __floats2bfloat162_rn(x.x > 0.f ? g.x : 0.f, x.y > 0.f ? g.y : 0.f);
    }
}

// out[j] += sum_r Y[r][j], j < 64 (bias and initial-vector gradients)
__global__ void colsum_kernel(const __nv_bfloat16 *Y, int ldy, int rows, float *out)
{
    const int lane = threadIdx.x & 31;
    float2 acc = make_float2(0.f, 0.f);
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += (gridDim.x * blockDim.x) >> 5) {
        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(Y + (size_t)r * ldy + 2 * lane));
        acc.x += f.x;
        acc.y += f.y;
    }
    atomicAdd(&out[2 * lane], acc.x);
    atomicAdd(&out[2 * lane + 1], acc.y);
}

// H[r] = vec (bf16), 64 channels
__global__ void broadcast_kernel(const float *vec, int rows, __nv_bfloat16 *H, int ldh)
{
    const int64_t total = (int64_t)rows * 32;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int c = 2 * (int)(t & 31);
        *reinterpret_cast<__nv_bfloat162 *>(H + (t >> 5) * ldh + c) = __floats2bfloat162_rn(vec[c], vec[c + 1]);
    }
}

// Heads and losses, one warp per variable row.
//   score = H . ws + bs  -> activity target y in [0, 1]: (sigmoid(score) - y)^2 * wa
//   phase = H . wp + bp  -> phase target t in {0, 1}:  BCE(sigmoid(phase), t) * wph
// head = [ws(64) | wp(64) | bs | bp]; grads accumulate into ghead (same layout);
// dH gets the gradient of the summed loss; loss[0..1] the two loss sums.
// Pass targets == null for inference: writes score and phase only.
__global__ void head_kernel(const __nv_bfloat16 *H, int ldh, int rows, const float *head, const float *y_act,
                            const float *w_act, const float *t_phase, const float *w_phase, float *score,
                            float *phase, __nv_bfloat16 *dH, int ldd, float *ghead, float *loss)
{
    const int lane = threadIdx.x & 31;
    const float ws0 = head[2 * lane], ws1 = head[2 * lane + 1];
    const float wp0 = head[64 + 2 * lane], wp1 = head[64 + 2 * lane + 1];
    const float bs = head[128], bp = head[129];
    float gs0 = 0.f, gs1 = 0.f, gp0 = 0.f, gp1 = 0.f, gbs = 0.f, gbp = 0.f, la = 0.f, lp = 0.f;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += (gridDim.x * blockDim.x) >> 5) {
        const float2 h = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(H + (size_t)r * ldh + 2 * lane));
        float s = h.x * ws0 + h.y * ws1, p = h.x * wp0 + h.y * wp1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            p += __shfl_xor_sync(0xffffffffu, p, o);
        }
        s += bs;
        p += bp;
        if (score && lane == 0) score[r] = s;
        if (phase && lane == 0) phase[r] = p;
        if (!y_act) continue;
        const float ps = 1.f / (1.f + __expf(-s)), pp = 1.f / (1.f + __expf(-p));
        const float wa = w_act[r], wph = w_phase[r];
        const float ds = 2.f * (ps - y_act[r]) * ps * (1.f - ps) * wa;
        const float dp = (pp - t_phase[r]) * wph;
        if (lane == 0) {
            la += (ps - y_act[r]) * (ps - y_act[r]) * wa;
            const float t = t_phase[r];
            lp += -(t * __logf(fmaxf(pp, 1e-12f)) + (1.f - t) * __logf(fmaxf(1.f - pp, 1e-12f))) * wph;
        }
        *reinterpret_cast<__nv_bfloat162 *>(dH + (size_t)r * ldd + 2 * lane) =
            __floats2bfloat162_rn(ds * ws0 + dp * wp0, ds * ws1 + dp * wp1);
        gs0 += ds * h.x;
        gs1 += ds * h.y;
        gp0 += dp * h.x;
        gp1 += dp * h.y;
        gbs += ds;
        gbp += dp;
    }
    if (!y_act) return;
    atomicAdd(&ghead[2 * lane], gs0);
    atomicAdd(&ghead[2 * lane + 1], gs1);
    atomicAdd(&ghead[64 + 2 * lane], gp0);
    atomicAdd(&ghead[64 + 2 * lane + 1], gp1);
    if (lane == 0) {
        atomicAdd(&ghead[128], gbs);
        atomicAdd(&ghead[129], gbp);
        atomicAdd(&loss[0], la);
        atomicAdd(&loss[1], lp);
    }
}

// Adam on fp32 parameters (bias-corrected), gradients zeroed afterwards.
__global__ void adam_kernel(float *p, float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        g[i] = 0.f;
    }
}

// W (K x N fp32, row-major) -> fwd = W^T (N x K bf16, dense) and bwd = W
// (K x N bf16, row stride ldb, so several maps can sit side by side)
__global__ void pack_kernel(const float *W, int K, int N, __nv_bfloat16 *fwd, __nv_bfloat16 *bwd, int ldb)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K * N; i += gridDim.x * blockDim.x) {
        const int k = i / N, n = i % N;
        const __nv_bfloat16 b = __float2bfloat16_rn(W[i]);
        if (bwd) bwd[(size_t)k * ldb + n] = b;
        if (fwd) fwd[(size_t)n * K + k] = b;
    }
}

}  // namespace gnn
}  // namespace gpsat

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace gpsat;

namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn()
{
    static std::once_flag once;
    static EncodeTiled fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    });
    return fn;
}

// a bf16 matrix of `rows` x `cols` (row stride `ld` elements), boxes of
// {8 elements, box_rows rows}
int make_map(CUtensorMap *m, const void *base, int64_t rows, int cols, int ld, int box_rows)
{
    EncodeTiled fn = encode_fn();
    if (!fn) return set_error(GPSAT_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    if (((uintptr_t)base & 15) || (ld * 2) % 16)
        return set_error(GPSAT_ERR_ARG, "gnn: matrices must be 16-byte aligned with 16-byte row strides");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GPSAT_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return GPSAT_OK;
}

int grid_for(int64_t work, int per_block)
{
    int64_t g = (work + per_block - 1) / per_block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

}  // namespace

extern "C" int gpsat_gnn_mm(const void *X, int32_t ldx, int64_t rows, int32_t K, const void *B, int32_t ldb,
                            int32_t N, const float *bias, int32_t relu, void *Y, int32_t ldy, int32_t *err,
                            void *stream)
{
    if (rows < 0 || rows > INT32_MAX || K <= 0 || K > gnn::MAXK || K % 64 || N <= 0 || N > gnn::MAXN || N % 64 ||
        ldx < K || ldb < K || ldy < N || (rows > 0 && (!X || !B || !Y || !err)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_mm: need K in {64,128,192}, N in {64,...,256}, ld >= width");
    if (rows == 0) return GPSAT_OK;
    if (((uintptr_t)Y & 15) || (ldy * 2) % 16) return set_error(GPSAT_ERR_ARG, "gpsat_gnn_mm: Y must be 16-byte aligned");
    CUtensorMap xm, bm;
    int rc = make_map(&xm, X, rows, K, ldx, gnn::TILE);
    if (rc == GPSAT_OK) rc = make_map(&bm, B, N, K, ldb, N);
    if (rc != GPSAT_OK) return rc;
    const size_t smem = (size_t)gnn::TILE * K * 2 + (size_t)N * K * 2 + 2 * 8 + 16;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(gnn::mm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(gnn::TILE * gnn::MAXK * 2 + gnn::MAXN * gnn::MAXK * 2 + 64));
    });
    if (attr != cudaSuccess) return cuda_error(attr, "gpsat_gnn_mm: shared memory attribute");
    gnn::MmArgs a{(int)rows, K, N, relu, bias, static_cast<__nv_bfloat16 *>(Y), ldy, err};
    gnn::mm_kernel<<<(unsigned)((rows + gnn::TILE - 1) / gnn::TILE), 128, smem, (cudaStream_t)stream>>>(xm, bm, a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_mm launch");
}

extern "C" int gpsat_gnn_wgrad(const void *X, int32_t ldx, const void *dY, int32_t ldy, int64_t rows, int32_t N,
                               float *dW, int32_t *err, void *stream)
{
    if (rows < 0 || rows > INT32_MAX || N <= 0 || N > gnn::WT_MAXN || N % 64 || ldx < 64 || ldy < N || ldx % 8 ||
        ldy % 8 || (rows > 0 && (!X || !dY || !dW)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_wgrad: need N in {64, 128, 192}, row strides multiples of 8");
    if (rows == 0) return GPSAT_OK;
    if (((uintptr_t)X & 15) || ((uintptr_t)dY & 15))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_wgrad: X and dY must be 16-byte aligned");
    const size_t smem = 2 * (size_t)128 * gnn::WT_R * 2 + 2 * (size_t)N * gnn::WT_R * 2 + 2 * 8 + 16;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(gnn::wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(2 * 128 * gnn::WT_R * 2 + 2 * gnn::WT_MAXN * gnn::WT_R * 2 + 64));
    });
    if (attr != cudaSuccess) return cuda_error(attr, "gpsat_gnn_wgrad: shared memory attribute");
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t chunks = (rows + gnn::WT_R - 1) / gnn::WT_R;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(chunks, sms));
    gnn::WgArgs a{static_cast<const __nv_bfloat16 *>(X), ldx, static_cast<const __nv_bfloat16 *>(dY), ldy,
                  (int)rows, N, dW, err};
    gnn::wgrad_kernel<<<grid, 128, smem, (cudaStream_t)stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_wgrad launch");
}

extern "C" int gpsat_gnn_gather(const int64_t *seg_off, const int32_t *edges, int64_t segs, const void *srcP,
                                const void *srcN, int32_t lds, const float *seg_scale, const void *Z, int32_t ldz,
                                void *out, int32_t ldo, int32_t relu, void *stream)
{
    if (segs < 0 || segs > INT32_MAX || (segs > 0 && (!seg_off || !srcP || !srcN || !out)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_gather: bad argument");
    if (segs == 0) return GPSAT_OK;
    gnn::gather_kernel<<<grid_for(segs * 32, 256), 256, 0, (cudaStream_t)stream>>>(
        seg_off, edges, (int)segs, static_cast<const __nv_bfloat16 *>(srcP), static_cast<const __nv_bfloat16 *>(srcN),
        lds, seg_scale, static_cast<const __nv_bfloat16 *>(Z), ldz, static_cast<__nv_bfloat16 *>(out), ldo, relu);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_gather launch");
}

extern "C" int gpsat_gnn_gather_split(const int64_t *seg_off, const int32_t *edges, int64_t segs, const void *src,
                                      int32_t lds, const float *src_scale, void *outP, void *outN, int32_t ldo,
                                      void *stream)
{
    if (segs < 0 || segs > INT32_MAX || (segs > 0 && (!seg_off || !src || !outP || !outN)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_gather_split: bad argument");
    if (segs == 0) return GPSAT_OK;
    gnn::gather_split_kernel<<<grid_for(segs * 32, 256), 256, 0, (cudaStream_t)stream>>>(
        seg_off, edges, (int)segs, static_cast<const __nv_bfloat16 *>(src), lds, src_scale,
        static_cast<__nv_bfloat16 *>(outP), static_cast<__nv_bfloat16 *>(outN), ldo);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_gather_split launch");
}

extern "C" int gpsat_gnn_relu_bwd(const void *dout, int32_t ldd, const void *h, int32_t ldh, int64_t rows, void *dpre,
                                  int32_t ldp, void *stream)
{
    if (rows < 0 || (rows > 0 && (!dout || !h || !dpre))) return set_error(GPSAT_ERR_ARG, "gpsat_gnn_relu_bwd");
    if (rows == 0) return GPSAT_OK;
    gnn::relu_bwd_kernel<<<grid_for(rows * 32, 256), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16 *>(dout), ldd, static_cast<const __nv_bfloat16 *>(h), ldh, (int)rows,
        static_cast<__nv_bfloat16 *>(dpre), ldp);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_relu_bwd launch");
}

extern "C" int gpsat_gnn_colsum(const void *Y, int32_t ldy, int64_t rows, float *out, void *stream)
{
    if (rows < 0 || (rows > 0 && (!Y || !out))) return set_error(GPSAT_ERR_ARG, "gpsat_gnn_colsum");
    if (rows == 0) return GPSAT_OK;
    gnn::colsum_kernel<<<std::min(grid_for(rows * 32, 256), 152 * 4), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16 *>(Y), ldy, (int)rows, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_colsum launch");
}

extern "C" int gpsat_gnn_broadcast(const float *vec, int64_t rows, void *H, int32_t ldh, void *stream)
{
    if (rows < 0 || (rows > 0 && (!vec || !H))) return set_error(GPSAT_ERR_ARG, "gpsat_gnn_broadcast");
    if (rows == 0) return GPSAT_OK;
    gnn::broadcast_kernel<<<grid_for(rows * 32, 256), 256, 0, (cudaStream_t)stream>>>(
        vec, (int)rows, static_cast<__nv_bfloat16 *>(H), ldh);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_broadcast launch");
}

extern "C" int gpsat_gnn_head(const void *H, int32_t ldh, int64_t rows, const float *head, const float *y_act,
                              const float *w_act, const float *t_phase, const float *w_phase, float *score,
                              float *phase, void *dH, int32_t ldd, float *ghead, float *loss, void *stream)
{
    if (rows < 0 || (rows > 0 && (!H || !head)) || (y_act && (!w_act || !t_phase || !w_phase || !dH || !ghead || !loss)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_head: bad argument");
    if (rows == 0) return GPSAT_OK;
    gnn::head_kernel<<<std::min(grid_for(rows * 32, 256), 152 * 8), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const __nv_bfloat16 *>(H), ldh, (int)rows, head, y_act, w_act, t_phase, w_phase, score, phase,
        static_cast<__nv_bfloat16 *>(dH), ldd, ghead, loss);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_head launch");
}

extern "C" int gpsat_gnn_adam(float *p, float *g, float *m, float *v, int64_t n, float lr, float beta1, float beta2,
                              float eps, int64_t step, void *stream)
{
    if (n < 0 || n > INT32_MAX || step <= 0 || (n > 0 && (!p || !g || !m || !v)))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_adam: bad argument");
    if (n == 0) return GPSAT_OK;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    gnn::adam_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, (int)n, lr, beta1, beta2, eps,
                                                                          c1, c2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_adam launch");
}

extern "C" int gpsat_gnn_pack(const float *W, int32_t K, int32_t N, void *fwd, void *bwd, int32_t ldb, void *stream)
{
    if (K <= 0 || N <= 0 || !W || (!fwd && !bwd) || (bwd && ldb < N))
        return set_error(GPSAT_ERR_ARG, "gpsat_gnn_pack: bad argument");
    gnn::pack_kernel<<<grid_for((int64_t)K * N, 256), 256, 0, (cudaStream_t)stream>>>(
        W, K, N, static_cast<__nv_bfloat16 *>(fwd), static_cast<__nv_bfloat16 *>(bwd), ldb);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPSAT_OK : cuda_error(e, "gpsat_gnn_pack launch");
}
