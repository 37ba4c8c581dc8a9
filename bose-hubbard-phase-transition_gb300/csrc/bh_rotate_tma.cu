// bh_rotate_tma.cu -- the thick-restart Ritz rotation of the FP32 Krylov basis
// on the 5th-generation tensor cores, with the basis streamed by TMA.
//
// The rotation  out_s[:, i] = sum_{c < kc} V_s[:, c] Y_s[c][i]  (M = D rows,
// K = kc basis vectors, N = nout kept Ritz vectors, one coefficient matrix
// Y_s per solve) of a whole batch whose solves all continue (input and output
// solve indices are the identity).  A CTA takes G = 8 / p adjacent solves
// (their columns of one basis row are 32 contiguous bytes) and a chunk of
// 128-row tiles.  Warp roles:
//   * warp 0, one lane: per K-step (8 basis vectors = 8/p blocks) one TMA box
//     {G p columns, 128 rows, 8/p blocks} into a ring of raw stages;
//   * warps 2..9 (thread = row and half of the CTA's solves): split each FP32
//     value x into two TF32 pieces x_hi = tf32(x), x_lo = tf32(x - x_hi) and
//     store both in tensor memory (tcgen05.st, lane = row, 8 columns of K;
//     ATM) or in shared memory in the UMMA K-major layout (core matrices of 8
//     rows x 16 bytes);
//   * warp 1, one lane: per K-step and solve the three products
//     x_hi y_hi + x_hi y_lo + x_lo y_hi as tcgen05.mma kind::tf32
//     M=128 x N=npad x K=8 into the solve's FP32 accumulator in tensor memory
//     (two accumulator sets, so a tile's products overlap the previous tile's
//     read-back);
//   * warps 10..13 (thread = row): read a finished tile's accumulators with
//     tcgen05.ld and write the G solves' outputs of one block of a row as two
//     16-byte stores.
// The dropped product x_lo y_lo and the rounding of the pieces leave a
// relative error of at most about 2^-22 per product term, below the FP32
// rounding of the accumulated sum.
// Ordering: every consumer thread releases a ring stage itself -- a raw stage
// after a proxy fence that orders its loads before the next TMA write -- and
// every converter thread publishes its own pieces (fence, then arrive); each
// K-step commits to one barrier (a tile's last step to the accumulator
// barrier, whose arrival then releases its operand stage); the MMA thread
// waits for its last commits before the CTA exits.  Every mbarrier wait is
// bounded: on a timeout the CTA records an error flag, every role stops, the
// producer and the MMA thread wait (bounded) for their operations in flight,
// and the tensor memory is freed.
#include <cuda.h>

#include <cstdint>

#include "bh_krylov.cuh"

namespace bh {

namespace {

constexpr int RT_M = 128;                 // rows per tile = tensor-memory lanes
constexpr int RT_KS = 8;                  // TF32 values per MMA K-step
constexpr int RT_THREADS = 448;           // 14 warps
constexpr unsigned RT_SPIN = 1u << 24;    // polls of an mbarrier before giving up
constexpr int RT_HEADER = 1024;           // bytes before the tiles (barriers, flags)
constexpr int RT_MAX_RAW = 6, RT_MAX_A = 2;
constexpr int RT_CONV = 256;              // converter threads (warps 2..9)

// Shared-memory header: barrier indices
enum : int {
    B_RAW_FULL = 0,                        // [RT_MAX_RAW]
    B_RAW_EMPTY = B_RAW_FULL + RT_MAX_RAW,  // [RT_MAX_RAW]
    B_A_FULL = B_RAW_EMPTY + RT_MAX_RAW,    // [RT_MAX_A]
    B_A_EMPTY = B_A_FULL + RT_MAX_A,        // [RT_MAX_A]
    B_ACC_FULL = B_A_EMPTY + RT_MAX_A,      // [2]
    B_ACC_EMPTY = B_ACC_FULL + 2,           // [2]
    B_COUNT = B_ACC_EMPTY + 2
};
constexpr int OFF_TMEM = B_COUNT * 8;      // uint32 tensor-memory address
constexpr int OFF_ERR = OFF_TMEM + 4;      // int error flag
constexpr int OFF_NRAW = OFF_ERR + 4;      // TMA loads issued (producer)
constexpr int OFF_NMMA = OFF_NRAW + 4;     // K-steps committed (MMA thread)
static_assert(OFF_NMMA + 4 <= RT_HEADER, "header");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of (row, k) in one K-step tile (K-major, no swizzle).
__device__ __forceinline__ uint32_t tile_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t tile_desc(uint32_t addr) {
    constexpr uint64_t lbo = 128 >> 4, sbo = 256 >> 4;
    return (uint64_t)((addr & 0x3FFFF) >> 4) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// x = hi + lo with hi = x rounded to TF32 and lo the (exact) rest rounded to
// TF32: |x - hi - lo| <= 2^-22 |x| (a truncated hi would give 2^-21), and the
// dropped product lo_a lo_b has no preferred sign
__device__ __forceinline__ void split2(float x, float& hi, float& lo) {
    hi = tf32_rna(x);
    lo = tf32_rna(x - hi);
}

// waits for the completion of the phase with this parity; false on timeout
// or when another role of the CTA has already given up
__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity, volatile int* err) {
    for (unsigned it = 0; it < RT_SPIN; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 1023) == 1023 && *err) return false;
    }
    *err = 1;
    return false;
}

// the n-th use of a ring slot: "full" barriers complete phase n, "empty"
// barriers start free (their phase -1 counts as complete)
__device__ __forceinline__ bool wait_full(uint32_t bar, int64_t use, volatile int* err) {
    return wait_parity(bar, (uint32_t)(use & 1), err);
}
__device__ __forceinline__ bool wait_empty(uint32_t bar, int64_t use, volatile int* err) {
    return wait_parity(bar, (uint32_t)((use & 1) ^ 1), err);
}

__device__ __forceinline__ void bar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// the same product with A read from tensor memory (lane = row, 8 columns of K)
__device__ __forceinline__ void mma_tf32_ta(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}" ::"r"(dtmem),
        "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 16 consecutive accumulator columns of this warp's 32 lanes; the caller waits
// (tmem_wait) before using them, so several loads share one wait
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace

// Shared memory (dynamic): header, B[g][piece][ks] coefficient tiles (npad
// rows x 32 bytes), raw[NR] TMA stages ({8/p blocks}[128 rows][8 floats]),
// A[NA][g][piece] operand tiles (128 rows x 32 bytes).
template <int P, bool ATM>
__global__ void __launch_bounds__(RT_THREADS, 1)
k_rotate_tma(const __grid_constant__ CUtensorMap tmap, int64_t D, int Sproc, int kc, int nout,
             const float* __restrict__ Yg, float* __restrict__ Vout, int64_t ostride, int ld_out, int npad,
             int nks, int NR, int NA, int tmem_cols, int64_t rows_per_cta, int* __restrict__ status) {
    constexpr int G = 8 / P;         // solves per CTA: G P = 8 columns = 32 bytes per row and block
    constexpr int KB = RT_KS / P;    // basis blocks per K-step
    constexpr int RAW = KB * RT_M * 32;
    constexpr int ATILE = RT_M * 32;
    extern __shared__ __align__(1024) unsigned char s_rt[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(s_rt);
    volatile int* err = reinterpret_cast<volatile int*>(s_rt + OFF_ERR);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int sg0 = blockIdx.x * G;
    const int nsg = min(G, Sproc - sg0);
    const int btile = npad * 32;
    unsigned char* sB = s_rt + RT_HEADER;
    unsigned char* sRaw = sB + (size_t)G * 2 * nks * btile;
    unsigned char* sA = sRaw + (size_t)NR * RAW;  // (ATM: the A stages are in tensor memory)
    auto bar = [&](int i) { return smem_u32(&bars[i]); };

    if (tid == 0) {
        for (int i = 0; i < NR; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(B_RAW_FULL + i)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(B_RAW_EMPTY + i)), "r"(RT_CONV));
        }
        for (int i = 0; i < NA; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(B_A_FULL + i)), "r"(RT_CONV));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(B_A_EMPTY + i)));
        }
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar(B_ACC_FULL + i)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(B_ACC_EMPTY + i)), "r"(RT_M));
        }
        *err = 0;
        *reinterpret_cast<volatile int*>(s_rt + OFF_NRAW) = 0;
        *reinterpret_cast<volatile int*>(s_rt + OFF_NMMA) = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(s_rt + OFF_TMEM)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // the G coefficient matrices, split into TF32 pieces (zero beyond kc, nout
    // and for the solves past the batch)
    const int kcp = nks * RT_KS;
    for (int e = tid; e < G * kcp * npad; e += blockDim.x) {
        const int g = e / (kcp * npad), rem = e - g * (kcp * npad);
        const int c = rem / npad, o = rem - c * npad;
        const float y = (g < nsg && c < kc && o < nout) ? Yg[((size_t)(sg0 + g) * kc + c) * nout + o] : 0.f;
        float y0, y1;
        split2(y, y0, y1);
        unsigned char* base = sB + ((size_t)(g * 2) * nks + c / RT_KS) * btile + tile_off(o, c & 7);
        *reinterpret_cast<float*>(base) = y0;
        *reinterpret_cast<float*>(base + (size_t)nks * btile) = y1;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(s_rt + OFF_TMEM);

    const int64_t r0 = (int64_t)blockIdx.y * rows_per_cta;
    const int64_t r1 = min(D, r0 + rows_per_cta);
    const int64_t ntile = r1 > r0 ? (r1 - r0 + RT_M - 1) / RT_M : 0;
    const int64_t nstep = ntile * nks;

    if (warp == 0) {
        // ---- producer: one TMA box per K-step ----
        if (lane == 0) {
            const uint64_t tm = reinterpret_cast<uint64_t>(&tmap);
            for (int64_t s = 0; s < nstep; ++s) {
                const int slot = (int)(s % NR);
                if (!wait_empty(bar(B_RAW_EMPTY + slot), s / NR, err)) break;
                const int64_t t = s / nks;
                const int ks = (int)(s - t * nks);
                const uint32_t fb = bar(B_RAW_FULL + slot);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(RAW)
                             : "memory");
                const int c0 = sg0 * P, c1 = (int)(r0 + t * RT_M), c2 = ks * KB;
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                    " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(sRaw + (size_t)slot * RAW)),
                    "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(fb)
                    : "memory");
                *reinterpret_cast<volatile int*>(s_rt + OFF_NRAW) = (int)(s + 1);
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(npad >> 3) << 17) |
                                   ((uint32_t)(RT_M >> 4) << 24);
            for (int64_t s = 0; s < nstep; ++s) {
                const int64_t t = s / nks;
                const int ks = (int)(s - t * nks);
                const int acc = (int)(t & 1);
                if (ks == 0 && !wait_empty(bar(B_ACC_EMPTY + acc), t >> 1, err)) break;
                const int slot = (int)(s % NA);
                if (!wait_full(bar(B_A_FULL + slot), s / NA, err)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int g = 0; g < nsg; ++g) {
                    const uint32_t b0 = smem_u32(sB + ((size_t)(g * 2) * nks + ks) * btile);
                    const uint32_t d = tmem + (uint32_t)((acc * G + g) * npad);
                    if constexpr (ATM) {
                        // A pieces: 8 columns each after the accumulators
                        const uint32_t a0 = tmem + (uint32_t)(2 * G * npad + ((slot * G + g) * 2) * 8);
                        mma_tf32_ta(d, a0, tile_desc(b0), idesc, ks > 0 ? 1u : 0u);                      // hi hi
                        mma_tf32_ta(d, a0, tile_desc(b0 + (uint32_t)(nks * btile)), idesc, 1u);          // hi lo
                        mma_tf32_ta(d, a0 + 8u, tile_desc(b0), idesc, 1u);                              // lo hi
                    } else {
                        const uint32_t a0 = smem_u32(sA + (size_t)(slot * G + g) * 2 * ATILE);
                        mma_tf32(d, tile_desc(a0), tile_desc(b0), idesc, ks > 0 ? 1u : 0u);              // hi hi
                        mma_tf32(d, tile_desc(a0), tile_desc(b0 + (uint32_t)(nks * btile)), idesc, 1u);  // hi lo
                        mma_tf32(d, tile_desc(a0 + ATILE), tile_desc(b0), idesc, 1u);                  // lo hi
                    }
                }
                if (ks != nks - 1) {
                    mma_commit(bar(B_A_EMPTY + slot));
                } else {
                    // A tile's last step commits to the accumulator barrier only:
                    // two commits with no product between them left the read-back
                    // reading a tile before its last products had landed.  Its
                    // operand slot is released once those products are complete.
                    mma_commit(bar(B_ACC_FULL + acc));
                    if (!wait_full(bar(B_ACC_FULL + acc), t >> 1, err)) break;
                    bar_arrive(bar(B_A_EMPTY + slot));
                }
                *reinterpret_cast<volatile int*>(s_rt + OFF_NMMA) = (int)(s + 1);
            }
            // The read-back waits for the accumulator commits only: the last
            // operand-slot commits must also have arrived before the CTA exits,
            // or their arrivals could land in the barriers of the next CTA on
            // this SM.
            for (int64_t s = nstep > NA ? nstep - NA : 0; s < nstep && !*err; ++s)
                (void)wait_full(bar(B_A_EMPTY + (int)(s % NA)), s / NA, err);
        }
    } else if (warp < 10) {
        // ---- converters: thread = row of the tile, warps 2..5 and 6..9 take
        // the first and second half of the CTA's solves ----
        constexpr int GH = G / 2;  // solves per converter thread
        // row in the warp's tensor-memory lane quarter (warp w reaches lanes
        // 32 (w % 4) .. + 31)
        const int row = (warp & 3) * 32 + lane;
        const int half = (warp - 2) >> 2;
        for (int64_t s = 0; s < nstep; ++s) {
            const int rs = (int)(s % NR);
            if (!wait_full(bar(B_RAW_FULL + rs), s / NR, err)) break;
            // this row's GH P values of each of the KB blocks: 16 bytes per block
            float x[KB][4];
            const unsigned char* raw = sRaw + (size_t)rs * RAW + (size_t)row * 32 + half * 16;
#pragma unroll
            for (int b = 0; b < KB; ++b) {
                const float4 u = *reinterpret_cast<const float4*>(raw + (size_t)b * RT_M * 32);
                x[b][0] = u.x; x[b][1] = u.y; x[b][2] = u.z; x[b][3] = u.w;
            }
            // the pieces of this thread's values, in registers before the slot is
            // released
            float hi[GH][8], lo[GH][8];
#pragma unroll
            for (int gg = 0; gg < GH; ++gg)
#pragma unroll
                for (int k = 0; k < 8; ++k)  // K index k = block (k / P), value k % P
                    split2(x[k / P][gg * P + k % P], hi[gg][k], lo[gg][k]);
            // The next TMA into this slot is an async-proxy write: every thread
            // orders its own shared-memory loads before it with a proxy fence and
            // releases the slot itself (an arrive alone, or one lane arriving for
            // the warp, let the TMA overwrite values still being loaded).
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bar_arrive(bar(B_RAW_EMPTY + rs));
            const int as = (int)(s % NA);
            if (!wait_empty(bar(B_A_EMPTY + as), s / NA, err)) break;
            if constexpr (ATM) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            unsigned char* aS = sA + (size_t)as * G * 2 * ATILE;
            const uint32_t o = tile_off(row, 0);
#pragma unroll
            for (int gg = 0; gg < GH; ++gg) {
                const int g = half * GH + gg;
                if constexpr (ATM) {
                    const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) +
                                        (uint32_t)(2 * G * npad + ((as * G + g) * 2) * 8);
                    tmem_st8(ta, hi[gg]);
                    tmem_st8(ta + 8u, lo[gg]);
                } else {
                    unsigned char* ah = aS + (size_t)g * 2 * ATILE + o;
                    *reinterpret_cast<float4*>(ah) = make_float4(hi[gg][0], hi[gg][1], hi[gg][2], hi[gg][3]);
                    *reinterpret_cast<float4*>(ah + 128) = make_float4(hi[gg][4], hi[gg][5], hi[gg][6], hi[gg][7]);
                    *reinterpret_cast<float4*>(ah + ATILE) = make_float4(lo[gg][0], lo[gg][1], lo[gg][2], lo[gg][3]);
                    *reinterpret_cast<float4*>(ah + ATILE + 128) =
                        make_float4(lo[gg][4], lo[gg][5], lo[gg][6], lo[gg][7]);
                }
            }
            // every thread makes its own writes visible to the products and
            // arrives itself
            if constexpr (ATM) {
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            } else {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            bar_arrive(bar(B_A_FULL + as));
        }
    } else {
        // ---- read-back: warp 10 + q reads tensor-memory lanes 32 ((10 + q) % 4) .. + 31 ----
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        for (int64_t t = 0; t < ntile; ++t) {
            const int acc = (int)(t & 1);
            if (!wait_full(bar(B_ACC_FULL + acc), t >> 1, err)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int64_t r = r0 + t * RT_M + row;
            const bool live = r < r1;
            // CW accumulator columns of every solve per chunk (8 when 8 solves
            // share the CTA, so that the chunk stays in registers)
            constexpr int CW = G > 4 ? 8 : 16;
            for (int c0 = 0; c0 < npad; c0 += CW) {
                uint32_t v[G][CW];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((acc * G + g) * npad + c0);
                    if constexpr (CW == 16) tmem_ld16(ta, v[g]);
                    else tmem_ld8(ta, v[g]);
                }
                tmem_wait();
                if (!live) continue;
                // outputs c0 .. c0 + CW - 1: blocks c0 / P ..; one block of a row
                // holds the G solves' P outputs, 8 contiguous floats
#pragma unroll
                for (int bb = 0; bb < CW / P; ++bb) {
                    const int i0 = c0 + bb * P;
                    if (i0 >= nout) break;
                    float w[8];
#pragma unroll
                    for (int g = 0; g < G; ++g)
#pragma unroll
                        for (int q = 0; q < P; ++q) w[g * P + q] = __uint_as_float(v[g][bb * P + q]);
                    float* dst = Vout + (int64_t)(i0 / P) * ostride + r * ld_out + (int64_t)sg0 * P;
                    if (nsg == G) {
                        reinterpret_cast<float4*>(dst)[0] = make_float4(w[0], w[1], w[2], w[3]);
                        reinterpret_cast<float4*>(dst)[1] = make_float4(w[4], w[5], w[6], w[7]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            if (e < nsg * P) dst[e] = w[e];
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            bar_arrive(bar(B_ACC_EMPTY + acc));
        }
    }

    // ---- teardown: nothing of this CTA may still be in flight ----
    __syncthreads();
    if (*err) {
        if (tid == 0 && status) atomicExch(status, 1);
        if (tid == 0) {
            // TMA loads issued: wait (bounded) for the last one of each slot
            const int nraw = *reinterpret_cast<volatile int*>(s_rt + OFF_NRAW);
            for (int i = 0; i < NR && i < nraw; ++i) {
                const int64_t last = nraw - 1 - i;  // the latest use of its slot
                for (unsigned it = 0; it < RT_SPIN; ++it) {
                    uint32_t done;
                    asm volatile(
                        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                        " selp.u32 %0, 1, 0, p;\n}"
                        : "=r"(done)
                        : "r"(bar(B_RAW_FULL + (int)(last % NR))), "r"((uint32_t)((last / NR) & 1))
                        : "memory");
                    if (done) break;
                }
            }
            // products committed: wait (bounded) for the last commit
            const int nmma = *reinterpret_cast<volatile int*>(s_rt + OFF_NMMA);
            if (nmma > 0) {
                const int64_t last = nmma - 1;
                for (unsigned it = 0; it < RT_SPIN; ++it) {
                    uint32_t done;
                    asm volatile(
                        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                        " selp.u32 %0, 1, 0, p;\n}"
                        : "=r"(done)
                        : "r"(bar(B_A_EMPTY + (int)(last % NA))), "r"((uint32_t)((last / NA) & 1))
                        : "memory");
                    if (done) break;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
}

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        (void)cudaGetLastError();
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

}  // namespace

bool rotate_tma(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride, const float* V,
                const float* Yg, float* Vout, int64_t ostride, int ld_out, int* d_status, cudaStream_t st,
                bool a_in_tmem) {
    if (Sproc <= 0 || D <= 0) return true;
    if (!(p == 1 || p == 2 || p == 4) || kc % p != 0 || kc <= 0) return false;
    const int G = 8 / p;
    const int npad = (nout + 15) / 16 * 16;
    if (2 * G * npad > 512) return false;  // two accumulator sets of G solves in 512 columns
    // 16-byte rules of the tensor map (base, strides) and of the 16-byte output stores
    if (((uintptr_t)V & 15) || ((uintptr_t)Vout & 15) || (ld_in * 4) % 16 || (bstride * 4) % 16 ||
        ld_out % 4 || (ostride * 4) % 16 || D > INT32_MAX)
        return false;
    const EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const int nks = (kc + RT_KS - 1) / RT_KS;
    const int KB = RT_KS / p;
    const size_t raw = (size_t)KB * RT_M * 32, atile = (size_t)RT_M * 32;
    const size_t bbytes = (size_t)G * 2 * nks * npad * 32;
    int smax = 0, dev = 0;
    BH_CUDA(cudaGetDevice(&dev));
    BH_CUDA(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int NR = RT_MAX_RAW, NA = RT_MAX_A;
    // A in tensor memory when its stages fit beside the two accumulator sets
    const bool atm = a_in_tmem && 2 * G * npad + NA * G * 16 <= 512;
    auto smem_of = [&]() {
        return (size_t)RT_HEADER + bbytes + NR * raw + (atm ? 0 : (size_t)NA * G * 2 * atile);
    };
    while (smem_of() > (size_t)smax && NR > 2) --NR;
    if (smem_of() > (size_t)smax) return false;
    // the CTA takes all 512 tensor-memory columns: enough shared memory that a
    // second CTA never shares its SM (its allocation would wait for this one)
    const size_t smem = std::max(smem_of(), std::min((size_t)smax, (size_t)120 * 1024));

    CUtensorMap tm;
    const cuuint64_t gdim[3] = {(cuuint64_t)ld_in, (cuuint64_t)D, (cuuint64_t)(kc / p)};
    const cuuint64_t gstride[2] = {(cuuint64_t)ld_in * 4, (cuuint64_t)bstride * 4};
    const cuuint32_t box[3] = {8u, (cuuint32_t)RT_M, (cuuint32_t)KB};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(V), gdim, gstride, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;

    const int ngroups = (Sproc + G - 1) / G;
    const int64_t tiles = (D + RT_M - 1) / RT_M;
    int64_t chunks = std::max<int64_t>(1, ((int64_t)2 * sm_count() + ngroups - 1) / ngroups);
    chunks = std::min(chunks, tiles);
    const int64_t tiles_per = (tiles + chunks - 1) / chunks;
    chunks = (tiles + tiles_per - 1) / tiles_per;
    if (chunks > 65535) return false;
    auto launch = [&](auto kern) {
        allow_large_smem(kern, smem);
        kern<<<dim3((unsigned)ngroups, (unsigned)chunks), RT_THREADS, smem, st>>>(
            tm, D, Sproc, kc, nout, Yg, Vout, ostride, ld_out, npad, nks, NR, NA, 512, tiles_per * RT_M, d_status);
    };
    if (atm) {
        if (p == 1) launch(k_rotate_tma<1, true>);
        else if (p == 2) launch(k_rotate_tma<2, true>);
        else launch(k_rotate_tma<4, true>);
    } else {
        if (p == 1) launch(k_rotate_tma<1, false>);
        else if (p == 2) launch(k_rotate_tma<2, false>);
        else launch(k_rotate_tma<4, false>);
    }
    BH_CUDA(cudaGetLastError());
    return true;
}

}  // namespace bh
