// K4: products with many right-hand sides through 16-bit tensor-core GEMMs.
//
//   YF = F X,  YG = G V      (N x R complex, R right-hand sides)
//
// The matrices are generated in row strips by the mixed-precision assembly
// (complex64, FP64 near pairs), each strip is quantised to 16-bit tiles and
// multiplied by all right-hand sides at once with tcgen05.mma (kind::f16,
// FP32 accumulator in tensor memory).  The reference forms the same products
// column batch by column batch through FMM3D (FMMFOperator / FMMGOperator
// `_unsafe_mul!` on a matrix, src/3d/fast_multipole_method.jl:249-287,
// 427-471).
//
// Complex GEMM as one real GEMM.  With K = 2N and the complex matrix stored
// with real and imaginary parts interleaved along K,
//   A[i][2j] = Re F_ij,  A[i][2j+1] = Im F_ij,
// and two real rows of the right-hand-side operand per column c,
//   B[c][2j] = Re X_jc,      B[c][2j+1] = -Im X_jc     -> (A B^T)[i][c]      = Re (F X)_ic
//   B[Rp+c][2j] = Im X_jc,   B[Rp+c][2j+1] = Re X_jc   -> (A B^T)[i][Rp + c] = Im (F X)_ic
// so a single M x 2Rp x 2N real GEMM (8 N^2 R flops) gives the product.
//
// Scaling.  Every row i of A carries a power of two 2^e_i chosen so that its
// largest component lands in [2^13, 2^14); every row of B (right-hand side c)
// likewise 2^f_c.  The scales factor out of the K sum and are applied in FP64
// when the partial sums are reduced, so FP16 never overflows and BF16 loses
// nothing.  Split precision adds lo parts: a = hi + lo with lo = q(a - hi), and
// A B^T ~ Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T, all three accumulated into the same
// FP32 tensor-memory tile.
//
// Operand layout in HBM ("tiled, 128-byte swizzled, K-major"): an operand with
// rows r and K columns is cut into tiles of RB rows (128 for A, 256 for B) by
// 64 K elements; the tiles of one row block are consecutive along K.  Inside a
// tile, row r occupies 128 bytes at r * 128 and its 16-byte chunk c (K elements
// 8c .. 8c+7) sits at chunk position c ^ (r & 7): the shared-memory image the
// tensor core reads with a SWIZZLE_128B K-major descriptor (8-row groups of
// 1024 bytes).  One bulk copy (cp.async.bulk) moves a whole tile into shared
// memory; no tensor map is needed.
//
// GEMM kernel (one CTA per 128 x 256 output tile and K range, 128 threads):
//   warp 0 lane 0: producer, bulk copies of the A and B tiles of each k-block
//                  into a ring of shared-memory stages (mbarrier full[s]);
//   warp 1 lane 0: issues tcgen05.mma (M=128, N=256, K=16) four times per
//                  k-block and term, then tcgen05.commit -> empty[s];
//   all 4 warps:   epilogue, tcgen05.ld of the FP32 accumulator (warp w owns
//                  tensor-memory lanes 32w .. 32w+31 = tile rows) and
//                  coalesced stores of the partial sums, column-major.
// Every mbarrier wait is bounded by a clock64 budget; a wait that gives up sets
// a bit in a device error word (reported as BIE_ERR_TIMEOUT), the CTA waits for
// its own MMAs and copies in flight (bounded again, with the long budget),
// frees its tensor memory and exits.  After the tensor-memory allocation no
// path returns before the deallocation.  The pipeline waits' budget is the
// context's (bie_ctx_set_gemm_wait), so a test can make one run out.
#include "bie_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace bie {

namespace {

constexpr int kBK = 64;                  // K elements per k-block (one 128-byte row)
constexpr int kBM = 128;                 // rows of an A tile = MMA M
constexpr int kBN = 256;                 // rows of a B tile  = MMA N
constexpr int kATile = kBM * 128;        // bytes of an A tile (16 KiB)
constexpr int kBTile = kBN * 128;        // bytes of a B tile (32 KiB)
constexpr int kGemmThreads = 128;
constexpr int kTmemCols = 256;           // FP32 accumulator columns (= kBN)
constexpr long long kWaitCycles = 4000000000LL;   // ~2 s at 2 GHz per wait
constexpr int kTargetExp = 14;           // row maxima scaled into [2^13, 2^14)

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and bit `code` set in *err) when `budget` clock cycles
// pass without the phase completing.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code,
                                          long long budget = kWaitCycles) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > budget) {
            atomicOr(err, 1 << code);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D[tmem] (+)= A[smem] . B[smem]^T, both K-major, 16-bit inputs, FP32 accumulator
__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
// arrive on `bar` once every previously issued tcgen05.mma of this thread completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
// 32 consecutive FP32 columns of the warp's 32 tensor-memory lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
          "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
          "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
          "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B
// apart (stride byte offset), leading byte offset unused for this layout,
// descriptor version 1, base offset 0 (tiles are 1024-byte aligned).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}
// Instruction descriptor of kind::f16: FP32 accumulator, A and B of one type
// (0 = F16, 1 = BF16), both K-major, N = 256, M = 128.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t bf16) {
    return (1u << 4) | (bf16 << 7) | (bf16 << 10) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

// ---------------------------------------------------------------------------
// The GEMM: P[ks][col][row] = sum over the split's K range of A[row] . B[col]
// ---------------------------------------------------------------------------
struct GemmArgs {
    const uint8_t *A[2];   // hi, lo tiles (lo unused unless split)
    const uint8_t *B[2];
    float *P;              // [ksplit][ncols_pad][mrows_pad]
    int64_t mrows_pad, ncols_pad;
    int nkb, kb_per;
    int *err;
    long long wait_cycles;   // budget of the pipeline waits (producer, MMA issuer)
    int stall;               // failure-detection test: the MMA issuer first waits on a
                             // barrier that nothing completes, so its wait runs out
};

template <int NT> struct StageShape {
    static constexpr int kBytes = NT * (kATile + kBTile);
};

template <bool BF, bool SPLIT, int STAGES>
__global__ void __launch_bounds__(kGemmThreads, 1) lowp_gemm_kernel(GemmArgs g) {
    constexpr int NT = SPLIT ? 2 : 1;   // hi (+ lo) tiles of each operand per stage
    constexpr int kStage = StageShape<NT>::kBytes;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * kStage);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint64_t *never = done + 1;   // completed by nothing (the stall test's wait)
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 2);
    __shared__ int s_issued, s_consumed;

    const int mb = blockIdx.x, nb = blockIdx.y, ks = blockIdx.z;
    const int kb0 = ks * g.kb_per;
    const int nit = min(g.nkb, kb0 + g.kb_per) - kb0;   // >= 1 by construction
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // a CTA of a launch in which another CTA already gave up does no work
    __shared__ int s_abort;
    if (threadIdx.x == 0) s_abort = *reinterpret_cast<volatile int *>(g.err);
    __syncthreads();
    if (s_abort) return;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        mbar_init(never, 1);
        s_issued = 0;
        s_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- producer ----
        int it = 0;
        for (; it < nit; ++it) {
            const int s = it % STAGES, n = it / STAGES;
            if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1, g.err, 0, g.wait_cycles)) break;
            mbar_expect_tx(&full[s], kStage);
            uint8_t *st = smem + (size_t)s * kStage;
            const int64_t kb = kb0 + it;
#pragma unroll
            for (int t = 0; t < NT; ++t)
                bulk_g2s(st + t * kATile, g.A[t] + ((int64_t)mb * g.nkb + kb) * kATile, kATile, &full[s]);
#pragma unroll
            for (int t = 0; t < NT; ++t)
                bulk_g2s(st + NT * kATile + t * kBTile, g.B[t] + ((int64_t)nb * g.nkb + kb) * kBTile, kBTile,
                         &full[s]);
        }
        s_issued = it;
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_f16(BF ? 1u : 0u);
        int it = 0;
        // stall test: a wait on a barrier that nothing completes runs out and
        // the issuer gives up before its first MMA, as after a lost copy
        if (g.stall) mbar_wait(never, 0, g.err, 4, g.wait_cycles);
        for (; !g.stall && it < nit; ++it) {
            const int s = it % STAGES, n = it / STAGES;
            if (!mbar_wait(&full[s], n & 1, g.err, 1, g.wait_cycles)) break;
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + (size_t)s * kStage);
            const uint32_t b0 = a0 + NT * kATile;
#pragma unroll
            for (int k = 0; k < kBK / 16; ++k) {   // K = 16 per instruction, 32 bytes
                const uint64_t da = sdesc_sw128(a0 + 32 * k), db = sdesc_sw128(b0 + 32 * k);
                mma_f16(tmem, da, db, idesc, (it > 0 || k > 0) ? 1u : 0u);
                if (SPLIT) {
                    const uint64_t dal = sdesc_sw128(a0 + kATile + 32 * k);
                    const uint64_t dbl = sdesc_sw128(b0 + kBTile + 32 * k);
                    mma_f16(tmem, da, dbl, idesc, 1u);
                    mma_f16(tmem, dal, db, idesc, 1u);
                }
            }
            mma_commit(&empty[s]);   // stage s free once these MMAs completed
        }
        s_consumed = it;
        mma_commit(done);            // all MMAs of this CTA completed
    }
    __syncwarp();

    // ---- epilogue: tensor memory -> partial sums (column-major, coalesced) ----
    bool ok = true;
    if (lane == 0) ok = mbar_wait(done, 0, g.err, 2);
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    tc_fence_after();
    if (ok) {
        const int row = warp * 32 + lane;
        float *out = g.P + ((int64_t)ks * g.ncols_pad + (int64_t)nb * kBN) * g.mrows_pad + (int64_t)mb * kBM + row;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < kBN; c0 += 32) {
            uint32_t v[32];
            tmem_ld32(tbase + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) out[(int64_t)(c0 + j) * g.mrows_pad] = __uint_as_float(v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    // drain copies that were issued but never consumed (only after a failed wait)
    if (threadIdx.x == 0) {
        for (int it = s_consumed; it < s_issued; ++it)
            if (!mbar_wait(&full[it % STAGES], (it / STAGES) & 1, g.err, 3)) break;
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

template <bool SPLIT> constexpr int stages() { return SPLIT ? 2 : 4; }
template <bool SPLIT> constexpr size_t gemm_smem() {
    return (size_t)stages<SPLIT>() * StageShape<SPLIT ? 2 : 1>::kBytes + 1024 +
           (2 * stages<SPLIT>() + 2) * sizeof(uint64_t) + 16;
}

// ---------------------------------------------------------------------------
// 16-bit quantisation
// ---------------------------------------------------------------------------
template <bool BF> __device__ __forceinline__ uint32_t q16(float x, float &back) {
    if (BF) {
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        back = __bfloat162float(h);
        return (uint32_t)__bfloat16_as_ushort(h);
    } else {
        const __half h = __float2half_rn(x);
        back = __half2float(h);
        return (uint32_t)__half_as_ushort(h);
    }
}
// 8 values -> hi (and lo) 16-byte chunks
template <bool BF, bool SPLIT> __device__ __forceinline__ void quant8(const float (&v)[8], uint4 &hi, uint4 &lo) {
    uint32_t h[8], l[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        float b;
        h[t] = q16<BF>(v[t], b);
        if (SPLIT) {
            float bl;
            l[t] = q16<BF>(v[t] - b, bl);   // v - b is exact in FP32
        } else {
            l[t] = 0;
        }
    }
    hi = make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
    lo = make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
}
// power-of-two exponent e with max * 2^-e in [2^13, 2^14) (max given as FP32 bits)
__device__ __forceinline__ int scale_exp_f32(uint32_t maxbits) {
    if (maxbits == 0) return 0;
    const int E = (int)((maxbits >> 23) & 0xffu) - 127;
    return max(-100, min(100, E + 1 - kTargetExp));
}
__device__ __forceinline__ int scale_exp_f64(unsigned long long maxbits) {
    if (maxbits == 0) return 0;
    const int E = (int)((maxbits >> 52) & 0x7ffull) - 1023;
    return max(-100, min(100, E + 1 - kTargetExp));
}
// swizzled position (in 16-byte units) of chunk c of row r inside a tile
__device__ __forceinline__ int swz16(int r, int c) { return r * 8 + (c ^ (r & 7)); }

// row maxima of a column-major complex64 strip (rows x ncols, leading dim ld)
__global__ void strip_rowmax_kernel(const float2 *__restrict__ S, int64_t ld, int64_t rows, int64_t ncols,
                                    int64_t cols_per, unsigned *__restrict__ rmax) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int64_t j0 = (int64_t)blockIdx.y * cols_per, j1 = min(ncols, j0 + cols_per);
    unsigned m = 0;
    for (int64_t j = j0; j < j1; ++j) {
        const float2 f = S[r + j * ld];
        m = max(m, max(__float_as_uint(fabsf(f.x)), __float_as_uint(fabsf(f.y))));
    }
    atomicMax(&rmax[r], m);
}

// A tiles of a strip: block (kb, mb) writes tile (mb, kb) through shared memory
template <bool BF, bool SPLIT>
__global__ void __launch_bounds__(256) pack_strip_kernel(const float2 *__restrict__ S, int64_t ld, int64_t rows,
                                                         int64_t ncols, const unsigned *__restrict__ rmax, int nkb,
                                                         uint4 *__restrict__ Ahi, uint4 *__restrict__ Alo) {
    __shared__ uint4 sh[SPLIT ? 2 : 1][kATile / 16];
    const int kb = blockIdx.x, mb = blockIdx.y;
    for (int t = threadIdx.x; t < kBM * 8; t += blockDim.x) {
        const int r = t % kBM, ch = t / kBM;   // rows fastest: coalesced strip reads
        const int64_t row = (int64_t)mb * kBM + r;
        float v[8];
        if (row < rows) {
            const float sc = ldexpf(1.0f, -scale_exp_f32(rmax[row]));
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t j = (int64_t)kb * (kBK / 2) + ch * 4 + q;
                const float2 f = j < ncols ? S[row + j * ld] : make_float2(0.f, 0.f);
                v[2 * q] = f.x * sc;
                v[2 * q + 1] = f.y * sc;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0.f;
        }
        uint4 hi, lo;
        quant8<BF, SPLIT>(v, hi, lo);
        sh[0][swz16(r, ch)] = hi;
        if (SPLIT) sh[SPLIT ? 1 : 0][swz16(r, ch)] = lo;
    }
    __syncthreads();
    const int64_t tile = ((int64_t)mb * nkb + kb) * (kATile / 16);
    for (int t = threadIdx.x; t < kATile / 16; t += blockDim.x) {
        Ahi[tile + t] = sh[0][t];
        if (SPLIT) Alo[tile + t] = sh[SPLIT ? 1 : 0][t];
    }
}

// column maxima of X (N x R complex128, column-major)
__global__ void rhs_colmax_kernel(const double2 *__restrict__ X, int64_t N, int64_t per,
                                  unsigned long long *__restrict__ cmax) {
    const int64_t c = blockIdx.y;
    const int64_t j0 = (int64_t)blockIdx.x * per, j1 = min(N, j0 + per);
    unsigned long long m = 0;
    for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        const double2 x = X[j + c * N];
        m = max(m, max((unsigned long long)__double_as_longlong(fabs(x.x)),
                       (unsigned long long)__double_as_longlong(fabs(x.y))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&cmax[c], m);
}

// B tiles of the right-hand sides: thread per (k-block, operand row, chunk)
template <bool BF, bool SPLIT>
__global__ void pack_rhs_kernel(const double2 *__restrict__ X, int64_t N, int64_t R, int64_t Rp,
                                const unsigned long long *__restrict__ cmax, int nkb, uint4 *__restrict__ Bhi,
                                uint4 *__restrict__ Blo) {
    const int64_t rows = 2 * Rp;
    const int64_t total = (int64_t)nkb * rows * 8;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int ch = (int)(idx & 7);
        const int64_t t2 = idx >> 3;
        const int64_t row = t2 % rows, kb = t2 / rows;
        const bool imag_row = row >= Rp;
        const int64_t c = imag_row ? row - Rp : row;
        double dv[8];
        const double sc = c < R ? ldexp(1.0, -scale_exp_f64(cmax[c])) : 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t j = kb * (kBK / 2) + ch * 4 + q;
            const double2 x = (c < R && j < N) ? X[j + c * N] : make_double2(0.0, 0.0);
            dv[2 * q] = (imag_row ? x.y : x.x) * sc;
            dv[2 * q + 1] = (imag_row ? x.x : -x.y) * sc;
        }
        // hi from the value, lo from the FP64 remainder
        uint32_t h[8], l[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            float b, bl;
            h[t] = q16<BF>((float)dv[t], b);
            l[t] = SPLIT ? q16<BF>((float)(dv[t] - (double)b), bl) : 0u;
        }
        const int64_t nbk = row / kBN;
        const int r = (int)(row % kBN);
        const int64_t tile = (nbk * nkb + kb) * (kBTile / 16);
        Bhi[tile + swz16(r, ch)] =
            make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
        if (SPLIT)
            Blo[tile + swz16(r, ch)] =
                make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
    }
}

// Y[(row0 + r) + c ldY] = 2^(e_r + f_c) (sum_ks P[ks][c][r] + i sum_ks P[ks][Rp + c][r])
__global__ void lowp_reduce_complex_kernel(const float *__restrict__ P, int ksplit, int64_t mrows_pad,
                                           int64_t ncols_pad, int64_t rows, int64_t R, int64_t Rp,
                                           const unsigned *__restrict__ rmax,
                                           const unsigned long long *__restrict__ cmax, int64_t ldY, int64_t row0,
                                           double2 *__restrict__ Y) {
    const int64_t total = rows * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx % rows, c = idx / rows;
        double re = 0.0, im = 0.0;
        for (int s = 0; s < ksplit; ++s) {
            re += (double)P[((int64_t)s * ncols_pad + c) * mrows_pad + r];
            im += (double)P[((int64_t)s * ncols_pad + Rp + c) * mrows_pad + r];
        }
        const double sc = ldexp(1.0, scale_exp_f32(rmax[r]) + scale_exp_f64(cmax[c]));
        Y[(row0 + r) + c * ldY] = make_double2(re * sc, im * sc);
    }
}

// ---- real GEMM building block (bie_lowp_gemm_device) ----------------------
__global__ void rowmax_rowmajor_kernel(const float *__restrict__ A, int64_t K, unsigned *__restrict__ rmax) {
    const int64_t r = blockIdx.x;
    unsigned m = 0;
    for (int64_t k = threadIdx.x; k < K; k += blockDim.x) m = max(m, __float_as_uint(fabsf(A[r * K + k])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&rmax[r], m);
}

template <bool BF, bool SPLIT>
__global__ void pack_rowmajor_kernel(const float *__restrict__ A, int64_t rows, int64_t K, int RB,
                                     const unsigned *__restrict__ rmax, int nkb, int64_t rows_pad,
                                     uint4 *__restrict__ Ohi, uint4 *__restrict__ Olo) {
    const int64_t total = rows_pad * nkb * 8;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int ch = (int)(idx & 7);
        const int64_t t2 = idx >> 3;
        const int64_t row = t2 % rows_pad, kb = t2 / rows_pad;
        float v[8];
        if (row < rows) {
            const float sc = ldexpf(1.0f, -scale_exp_f32(rmax[row]));
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t k = kb * kBK + ch * 8 + q;
                v[q] = k < K ? A[row * K + k] * sc : 0.f;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0.f;
        }
        uint4 hi, lo;
        quant8<BF, SPLIT>(v, hi, lo);
        const int64_t tile = ((row / RB) * nkb + kb) * ((int64_t)RB * 8);
        const int r = (int)(row % RB);
        Ohi[tile + swz16(r, ch)] = hi;
        if (SPLIT) Olo[tile + swz16(r, ch)] = lo;
    }
}

__global__ void lowp_reduce_real_kernel(const float *__restrict__ P, int ksplit, int64_t mrows_pad,
                                        int64_t ncols_pad, int64_t M, int64_t N, const unsigned *__restrict__ ra,
                                        const unsigned *__restrict__ rb, double *__restrict__ C) {
    const int64_t total = M * N;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % M, j = idx / M;
        double s = 0.0;
        for (int t = 0; t < ksplit; ++t) s += (double)P[((int64_t)t * ncols_pad + j) * mrows_pad + i];
        C[i * N + j] = s * ldexp(1.0, scale_exp_f32(ra[i]) + scale_exp_f32(rb[j]));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Format {
    bool bf16, split;
};
Format format_of(int precision) {
    switch (precision) {
    case BIE_PREC_FP16: return {false, false};
    case BIE_PREC_BF16: return {true, false};
    case BIE_PREC_FP16_SPLIT: return {false, true};
    case BIE_PREC_BF16_SPLIT: return {true, true};
    default: fail(BIE_ERR_INVALID, "not a 16-bit tensor-core precision: " + std::to_string(precision));
    }
}

inline unsigned grid1(int64_t n, int t = 256) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, 1 << 20));
}

template <bool BF, bool SPLIT> void set_gemm_attr() {
    BIE_CUDA(cudaFuncSetAttribute(lowp_gemm_kernel<BF, SPLIT, stages<SPLIT>()>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem<SPLIT>()));
}

// K split: enough CTAs to cover the SMs (but >= 8 k-blocks per split where
// possible), and at most kMaxKbPerSplit k-blocks (4096 K) summed in one FP32
// accumulator, so that rounding in the accumulator stays ~1e-6 relative; the
// partial sums are added in FP64.
// The limit can be lowered with the environment variable BIE_LOWP_MAX_KB
// (k-blocks of 64) to trade partial-sum traffic for accuracy.
int max_kb_per_split() {
    static const int v = [] {
        const char *e = std::getenv("BIE_LOWP_MAX_KB");
        const int x = e ? std::atoi(e) : 0;
        return x > 0 ? x : 64;
    }();
    return v;
}
void choose_split(const Ctx &c, int64_t mt, int64_t nt, int nkb, int &ksplit, int &kb_per) {
    const int64_t ctas = mt * nt;
    int64_t want = std::max<int64_t>(1, (c.num_sms + ctas - 1) / ctas);
    want = std::min<int64_t>(want, std::max(1, nkb / 8));
    const int maxkb = max_kb_per_split();
    want = std::max<int64_t>(want, (nkb + maxkb - 1) / maxkb);
    kb_per = (int)((nkb + want - 1) / want);
    ksplit = (nkb + kb_per - 1) / kb_per;
}

void launch_gemm(Ctx &c, Format f, const uint8_t *Ahi, const uint8_t *Alo, const uint8_t *Bhi,
                 const uint8_t *Blo, int64_t mt, int64_t nt, int nkb, int ksplit, int kb_per, float *P, int *err,
                 double algorithmic_flops) {
    GemmArgs g{};
    g.A[0] = Ahi;
    g.A[1] = Alo ? Alo : Ahi;
    g.B[0] = Bhi;
    g.B[1] = Blo ? Blo : Bhi;
    g.P = P;
    g.mrows_pad = mt * kBM;
    g.ncols_pad = nt * kBN;
    g.nkb = nkb;
    g.kb_per = kb_per;
    g.err = err;
    g.wait_cycles = c.gemm_wait_cycles < 0 ? kWaitCycles : (long long)c.gemm_wait_cycles;
    g.stall = c.gemm_stall ? 1 : 0;
    if (mt > 0x7fffffff || nt > 65535 || ksplit > 65535) fail(BIE_ERR_INVALID, "GEMM grid too large");
    dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)ksplit);
    const double executed = 2.0 * (double)(mt * kBM) * (double)(nt * kBN) * (double)nkb * kBK * (f.split ? 3 : 1);
    cudaEvent_t t0 = c.timing ? c.take_event() : nullptr;
    if (t0) BIE_CUDA(cudaEventRecord(t0, c.stream));
    if (f.bf16) {
        if (f.split) {
            set_gemm_attr<true, true>();
            lowp_gemm_kernel<true, true, stages<true>()><<<grid, kGemmThreads, gemm_smem<true>(), c.stream>>>(g);
        } else {
            set_gemm_attr<true, false>();
            lowp_gemm_kernel<true, false, stages<false>()><<<grid, kGemmThreads, gemm_smem<false>(), c.stream>>>(g);
        }
    } else {
        if (f.split) {
            set_gemm_attr<false, true>();
            lowp_gemm_kernel<false, true, stages<true>()><<<grid, kGemmThreads, gemm_smem<true>(), c.stream>>>(g);
        } else {
            set_gemm_attr<false, false>();
            lowp_gemm_kernel<false, false, stages<false>()><<<grid, kGemmThreads, gemm_smem<false>(), c.stream>>>(g);
        }
    }
    BIE_CUDA(cudaGetLastError());
    c.tensor_timer_end(t0, algorithmic_flops, executed);
    ++c.kernel_launches;
}

void check_err_word(Ctx &c, const int *d_err) {
    int h = 0;
    BIE_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    BIE_CUDA(cudaStreamSynchronize(c.stream));
    if (h) fail(BIE_ERR_TIMEOUT, "tensor-core GEMM wait gave up (code " + std::to_string(h) + ")");
}

// a carve-out allocator over one scratch slot
struct Carve {
    char *base;
    size_t off = 0;
    template <typename T> T *take(size_t bytes) {
        T *p = reinterpret_cast<T *>(base + off);
        off += (bytes + 1023) & ~size_t(1023);
        return p;
    }
};

template <bool BF, bool SPLIT>
void pack_strip(Ctx &c, const float2 *S, int64_t ld, int64_t rows, int64_t ncols, const unsigned *rmax, int nkb,
                int64_t mt, uint8_t *Ahi, uint8_t *Alo) {
    dim3 grid((unsigned)nkb, (unsigned)mt);
    pack_strip_kernel<BF, SPLIT><<<grid, 256, 0, c.stream>>>(S, ld, rows, ncols, rmax, nkb,
                                                             reinterpret_cast<uint4 *>(Ahi),
                                                             reinterpret_cast<uint4 *>(Alo));
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

void pack_strip_any(Ctx &c, Format f, const float2 *S, int64_t ld, int64_t rows, int64_t ncols,
                    const unsigned *rmax, int nkb, int64_t mt, uint8_t *Ahi, uint8_t *Alo) {
    if (f.bf16) {
        if (f.split) pack_strip<true, true>(c, S, ld, rows, ncols, rmax, nkb, mt, Ahi, Alo);
        else pack_strip<true, false>(c, S, ld, rows, ncols, rmax, nkb, mt, Ahi, Alo);
    } else {
        if (f.split) pack_strip<false, true>(c, S, ld, rows, ncols, rmax, nkb, mt, Ahi, Alo);
        else pack_strip<false, false>(c, S, ld, rows, ncols, rmax, nkb, mt, Ahi, Alo);
    }
}

void pack_rhs_any(Ctx &c, Format f, const double2 *X, int64_t N, int64_t R, int64_t Rp,
                  const unsigned long long *cmax, int nkb, uint8_t *Bhi, uint8_t *Blo) {
    const unsigned grid = grid1((int64_t)nkb * 2 * Rp * 8);
    uint4 *h = reinterpret_cast<uint4 *>(Bhi), *l = reinterpret_cast<uint4 *>(Blo);
    if (f.bf16) {
        if (f.split) pack_rhs_kernel<true, true><<<grid, 256, 0, c.stream>>>(X, N, R, Rp, cmax, nkb, h, l);
        else pack_rhs_kernel<true, false><<<grid, 256, 0, c.stream>>>(X, N, R, Rp, cmax, nkb, h, l);
    } else {
        if (f.split) pack_rhs_kernel<false, true><<<grid, 256, 0, c.stream>>>(X, N, R, Rp, cmax, nkb, h, l);
        else pack_rhs_kernel<false, false><<<grid, 256, 0, c.stream>>>(X, N, R, Rp, cmax, nkb, h, l);
    }
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

void pack_rowmajor_any(Ctx &c, Format f, const float *A, int64_t rows, int64_t K, int RB, const unsigned *rmax,
                       int nkb, int64_t rows_pad, uint8_t *Ohi, uint8_t *Olo) {
    const unsigned grid = grid1(rows_pad * nkb * 8);
    uint4 *h = reinterpret_cast<uint4 *>(Ohi), *l = reinterpret_cast<uint4 *>(Olo);
    if (f.bf16) {
        if (f.split)
            pack_rowmajor_kernel<true, true><<<grid, 256, 0, c.stream>>>(A, rows, K, RB, rmax, nkb, rows_pad, h, l);
        else
            pack_rowmajor_kernel<true, false><<<grid, 256, 0, c.stream>>>(A, rows, K, RB, rmax, nkb, rows_pad, h, l);
    } else {
        if (f.split)
            pack_rowmajor_kernel<false, true><<<grid, 256, 0, c.stream>>>(A, rows, K, RB, rmax, nkb, rows_pad, h, l);
        else
            pack_rowmajor_kernel<false, false><<<grid, 256, 0, c.stream>>>(A, rows, K, RB, rmax, nkb, rows_pad, h,
                                                                            l);
    }
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

}  // namespace

// ---------------------------------------------------------------------------
void run_lowp_gemm(Ctx &c, int precision, int64_t M, int64_t N, int64_t K, const float *A, const float *B,
                   double *C) {
    const Format f = format_of(precision);
    if (M <= 0 || N <= 0 || K <= 0) fail(BIE_ERR_INVALID, "GEMM sizes must be positive");
    const int64_t mt = (M + kBM - 1) / kBM, nt = (N + kBN - 1) / kBN;
    const int64_t nkb64 = (K + kBK - 1) / kBK;
    if (nkb64 > (1 << 30)) fail(BIE_ERR_INVALID, "K too large");
    const int nkb = (int)nkb64;
    int ksplit, kb_per;
    choose_split(c, mt, nt, nkb, ksplit, kb_per);
    const int nparts = f.split ? 2 : 1;
    const size_t abytes = (size_t)mt * nkb * kATile, bbytes = (size_t)nt * nkb * kBTile;
    const size_t pbytes = (size_t)ksplit * nt * kBN * mt * kBM * sizeof(float);
    const size_t total = nparts * (abytes + bbytes) + pbytes + (size_t)(M + N) * 4 + 4096 + 8 * 1024;
    Carve cv{static_cast<char *>(c.scratch(kScratchLowp, total))};
    uint8_t *Ahi = cv.take<uint8_t>(abytes), *Alo = f.split ? cv.take<uint8_t>(abytes) : nullptr;
    uint8_t *Bhi = cv.take<uint8_t>(bbytes), *Blo = f.split ? cv.take<uint8_t>(bbytes) : nullptr;
    float *P = cv.take<float>(pbytes);
    unsigned *ra = cv.take<unsigned>((size_t)M * 4), *rb = cv.take<unsigned>((size_t)N * 4);
    int *err = cv.take<int>(sizeof(int));
    BIE_CUDA(cudaMemsetAsync(ra, 0, (size_t)M * 4, c.stream));
    BIE_CUDA(cudaMemsetAsync(rb, 0, (size_t)N * 4, c.stream));
    BIE_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    rowmax_rowmajor_kernel<<<(unsigned)M, 256, 0, c.stream>>>(A, K, ra);
    rowmax_rowmajor_kernel<<<(unsigned)N, 256, 0, c.stream>>>(B, K, rb);
    BIE_CUDA(cudaGetLastError());
    c.kernel_launches += 2;
    pack_rowmajor_any(c, f, A, M, K, kBM, ra, nkb, mt * kBM, Ahi, Alo);
    pack_rowmajor_any(c, f, B, N, K, kBN, rb, nkb, nt * kBN, Bhi, Blo);
    launch_gemm(c, f, Ahi, Alo, Bhi, Blo, mt, nt, nkb, ksplit, kb_per, P, err, 2.0 * (double)M * N * K);
    lowp_reduce_real_kernel<<<grid1(M * N), 256, 0, c.stream>>>(P, ksplit, mt * kBM, nt * kBN, M, N, ra, rb, C);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
    check_err_word(c, err);
}

void run_matvec_multi(Ctx &c, const MultiArgs &a) {
    const int64_t N = c.n_sources, R = a.nrhs;
    if (a.precision == BIE_PREC_FP64 || a.precision == BIE_PREC_MIXED) {
        // one matrix-free product per column
        for (int64_t col = 0; col < R; ++col) {
            MatvecArgs m{a.k_re, a.k_im, c.d_sources, N,
                         a.X ? a.X + 2 * N * col : nullptr, a.V ? a.V + 2 * N * col : nullptr,
                         a.YF ? a.YF + 2 * N * col : nullptr, a.YG ? a.YG + 2 * N * col : nullptr,
                         a.precision};
            launch_matvec(c, m);
        }
        return;
    }
    const Format f = format_of(a.precision);
    const bool doF = a.X != nullptr, doG = a.V != nullptr;
    if (!doF && !doG) return;
    const int64_t Rp = (R + 127) / 128 * 128;
    const int64_t nt = 2 * Rp / kBN;
    const int64_t K = 2 * N;
    const int nkb = (int)((K + kBK - 1) / kBK);
    const int nparts = f.split ? 2 : 1;
    const int nops = (doF ? 1 : 0) + (doG ? 1 : 0);

    // strip height: complex64 strips of the requested matrices + their tiles
    const size_t budget = a.scratch_bytes > 0 ? (size_t)a.scratch_bytes : ((size_t)8 << 30);
    const size_t per_row = (size_t)nops * N * 8 + (size_t)nparts * nkb * kBK * 2;
    int64_t Ms = (int64_t)(budget / std::max<size_t>(per_row, 1)) / kBM * kBM;
    Ms = std::max<int64_t>(kBM, std::min<int64_t>(Ms, (N + kBM - 1) / kBM * kBM));
    const int64_t mt_max = Ms / kBM;
    int ksplit_max = 1, kb_per_dummy;
    choose_split(c, 1, nt, nkb, ksplit_max, kb_per_dummy);   // the largest split any strip uses

    const size_t strip_bytes = (size_t)Ms * N * 8;
    const size_t abytes = (size_t)mt_max * nkb * kATile;
    const size_t bbytes = (size_t)nt * nkb * kBTile;
    const size_t pbytes = (size_t)ksplit_max * nt * kBN * Ms * sizeof(float);
    const size_t total = nops * (strip_bytes + nparts * bbytes + 8 * 1024) + nparts * abytes + pbytes +
                         (size_t)Ms * 4 + (size_t)nops * R * 8 + 16 * 1024;
    Carve cv{static_cast<char *>(c.scratch(kScratchLowp, total))};
    float2 *SF = doF ? cv.take<float2>(strip_bytes) : nullptr;
    float2 *SG = doG ? cv.take<float2>(strip_bytes) : nullptr;
    uint8_t *BFh = doF ? cv.take<uint8_t>(bbytes) : nullptr;
    uint8_t *BFl = doF && f.split ? cv.take<uint8_t>(bbytes) : nullptr;
    uint8_t *BGh = doG ? cv.take<uint8_t>(bbytes) : nullptr;
    uint8_t *BGl = doG && f.split ? cv.take<uint8_t>(bbytes) : nullptr;
    uint8_t *Ahi = cv.take<uint8_t>(abytes), *Alo = f.split ? cv.take<uint8_t>(abytes) : nullptr;
    float *P = cv.take<float>(pbytes);
    unsigned *rmax = cv.take<unsigned>((size_t)Ms * 4);
    unsigned long long *cmF = doF ? cv.take<unsigned long long>((size_t)R * 8) : nullptr;
    unsigned long long *cmG = doG ? cv.take<unsigned long long>((size_t)R * 8) : nullptr;
    int *err = cv.take<int>(sizeof(int));
    BIE_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));

    // right-hand-side operands, once per call
    const int64_t cper = 4096;
    auto prep_rhs = [&](const double *Xd, unsigned long long *cm, uint8_t *Bh, uint8_t *Bl) {
        BIE_CUDA(cudaMemsetAsync(cm, 0, (size_t)R * 8, c.stream));
        dim3 g((unsigned)((N + cper - 1) / cper), (unsigned)R);
        rhs_colmax_kernel<<<g, 256, 0, c.stream>>>(reinterpret_cast<const double2 *>(Xd), N, cper, cm);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        pack_rhs_any(c, f, reinterpret_cast<const double2 *>(Xd), N, R, Rp, cm, nkb, Bh, Bl);
    };
    if (R > 65535) fail(BIE_ERR_INVALID, "at most 65535 right-hand sides per call");
    if (doF) prep_rhs(a.X, cmF, BFh, BFl);
    if (doG) prep_rhs(a.V, cmG, BGh, BGl);

    for (int64_t i0 = 0; i0 < N; i0 += Ms) {
        const int64_t ms = std::min<int64_t>(Ms, N - i0);
        const int64_t mt = (ms + kBM - 1) / kBM;
        AssembleArgs s{a.k_re, a.k_im, c.d_sources + 3 * i0, ms, (doF ? BIE_F : 0) | (doG ? BIE_G : 0),
                       reinterpret_cast<double *>(SF), reinterpret_cast<double *>(SG), nullptr};
        s.c64_out = true;
        launch_assemble_mixed(c, s);
        int ksplit, kb_per;
        choose_split(c, mt, nt, nkb, ksplit, kb_per);
        for (int op = 0; op < 2; ++op) {
            const float2 *S = op == 0 ? SF : SG;
            if (!S) continue;
            const unsigned long long *cm = op == 0 ? cmF : cmG;
            BIE_CUDA(cudaMemsetAsync(rmax, 0, (size_t)ms * 4, c.stream));
            const int64_t cols_per = 64;   // column blocks per strip: enough blocks in flight
            dim3 g((unsigned)((ms + 255) / 256), (unsigned)((N + cols_per - 1) / cols_per));
            strip_rowmax_kernel<<<g, 256, 0, c.stream>>>(S, ms, ms, N, cols_per, rmax);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
            pack_strip_any(c, f, S, ms, ms, N, rmax, nkb, mt, Ahi, Alo);
            launch_gemm(c, f, Ahi, Alo, op == 0 ? BFh : BGh, op == 0 ? BFl : BGl, mt, nt, nkb, ksplit, kb_per, P,
                        err, 8.0 * (double)ms * N * R);
            double2 *Y = reinterpret_cast<double2 *>(op == 0 ? a.YF : a.YG);
            lowp_reduce_complex_kernel<<<grid1(ms * R), 256, 0, c.stream>>>(P, ksplit, mt * kBM, nt * kBN, ms, R, Rp,
                                                                            rmax, cm, N, i0, Y);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
        }
    }
    check_err_word(c, err);
}

// ---------------------------------------------------------------------------
// A complex64 N x N matrix quantised once to resident 16-bit tiles, applied to
// blocks of right-hand sides (the inner products of the multi-RHS solve)
// ---------------------------------------------------------------------------
struct LowpMatrix {
    Format f{};
    int64_t n = 0, mt = 0;
    int nkb = 0;
    uint8_t *Ahi = nullptr, *Alo = nullptr;
    unsigned *rmax = nullptr;
    char *work = nullptr;   // B tiles, partial sums, column maxima, error word (grow-only)
    size_t work_bytes = 0;
};

LowpMatrix *lowp_matrix_create(Ctx &c, const float *A, int64_t n, int precision) {
    auto *m = new LowpMatrix();
    try {
        m->f = format_of(precision);
        m->n = n;
        m->mt = (n + kBM - 1) / kBM;
        const int64_t nkb64 = (2 * n + kBK - 1) / kBK;
        if (nkb64 > (1 << 30) || m->mt > 65535) fail(BIE_ERR_INVALID, "matrix too large for the tensor-core tiles");
        m->nkb = (int)nkb64;
        const size_t abytes = (size_t)m->mt * m->nkb * kATile;
        BIE_CUDA(cudaMalloc(&m->Ahi, abytes));
        if (m->f.split) BIE_CUDA(cudaMalloc(&m->Alo, abytes));
        BIE_CUDA(cudaMalloc(&m->rmax, (size_t)n * 4));
        BIE_CUDA(cudaMemsetAsync(m->rmax, 0, (size_t)n * 4, c.stream));
        const float2 *S = reinterpret_cast<const float2 *>(A);
        const int64_t cols_per = 64;   // column blocks per strip: enough blocks in flight
        dim3 g((unsigned)((n + 255) / 256), (unsigned)((n + cols_per - 1) / cols_per));
        strip_rowmax_kernel<<<g, 256, 0, c.stream>>>(S, n, n, n, cols_per, m->rmax);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        pack_strip_any(c, m->f, S, n, n, n, m->rmax, m->nkb, m->mt, m->Ahi, m->Alo);
    } catch (...) {
        lowp_matrix_destroy(m);
        throw;
    }
    return m;
}

void lowp_matrix_destroy(LowpMatrix *m) {
    if (!m) return;
    cudaFree(m->Ahi);
    cudaFree(m->Alo);
    cudaFree(m->rmax);
    cudaFree(m->work);
    delete m;
}

// Y = A X for X, Y: n x R complex128 (column-major, device)
void lowp_matrix_apply(Ctx &c, LowpMatrix &m, const double *X, int64_t R, double *Y) {
    if (R <= 0) return;
    if (R > 65535) fail(BIE_ERR_INVALID, "at most 65535 right-hand sides per product");
    const int64_t Rp = (R + 127) / 128 * 128;
    const int64_t nt = 2 * Rp / kBN;
    int ksplit, kb_per;
    choose_split(c, m.mt, nt, m.nkb, ksplit, kb_per);
    const int nparts = m.f.split ? 2 : 1;
    const size_t bbytes = (size_t)nt * m.nkb * kBTile;
    const size_t pbytes = (size_t)ksplit * nt * kBN * m.mt * kBM * sizeof(float);
    auto up = [](size_t b) { return (b + 1023) & ~size_t(1023); };
    const size_t need = nparts * up(bbytes) + up(pbytes) + up((size_t)R * 8) + up(sizeof(int));
    if (m.work_bytes < need) {
        if (c.capturing) fail(BIE_ERR_INVALID, "device scratch would grow while a CUDA graph is recorded");
        cudaFree(m.work);
        m.work = nullptr;
        m.work_bytes = 0;
        BIE_CUDA(cudaMalloc(&m.work, need));
        m.work_bytes = need;
    }
    Carve cv{m.work};
    uint8_t *Bh = cv.take<uint8_t>(bbytes), *Bl = m.f.split ? cv.take<uint8_t>(bbytes) : nullptr;
    float *P = cv.take<float>(pbytes);
    unsigned long long *cm = cv.take<unsigned long long>((size_t)R * 8);
    int *err = cv.take<int>(sizeof(int));
    BIE_CUDA(cudaMemsetAsync(cm, 0, (size_t)R * 8, c.stream));
    BIE_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    const int64_t cper = 4096;
    const double2 *Xd = reinterpret_cast<const double2 *>(X);
    dim3 g((unsigned)((m.n + cper - 1) / cper), (unsigned)R);
    rhs_colmax_kernel<<<g, 256, 0, c.stream>>>(Xd, m.n, cper, cm);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
    pack_rhs_any(c, m.f, Xd, m.n, R, Rp, cm, m.nkb, Bh, Bl);
    launch_gemm(c, m.f, m.Ahi, m.Alo, Bh, Bl, m.mt, nt, m.nkb, ksplit, kb_per, P, err,
                8.0 * (double)m.n * m.n * R);
    lowp_reduce_complex_kernel<<<grid1(m.n * R), 256, 0, c.stream>>>(P, ksplit, m.mt * kBM, nt * kBN, m.n, R, Rp,
                                                                     m.rmax, cm, m.n, 0,
                                                                     reinterpret_cast<double2 *>(Y));
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
    check_err_word(c, err);
}

}  // namespace bie
