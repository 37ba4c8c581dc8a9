// bh_rotate_tc.cu -- the thick-restart Ritz rotation of the FP32 Krylov basis
// on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory).
//
// The rotation  out_s[:, i] = sum_{c < kc} V_s[:, c] Y_s[c][i]  of every
// processed solve s is a dense product (M = D rows, K = kc basis vectors,
// N = nout outputs) with one small coefficient matrix per solve.  A CTA takes
// G solves and a chunk of rows, keeps the G coefficient matrices in shared
// memory for all of its row tiles, and per tile of 128 rows streams the basis
// through shared memory one K-step (8 basis vectors) at a time:
//   * every thread loads its row's 8 values per solve, splits each FP32 value
//     x into three TF32 pieces x0 + x1 + x2 (x0 = tf32(x), x1 = tf32(x - x0),
//     x2 = tf32(x - x0 - x1); 33 mantissa bits, so the split is exact) and
//     stores them in the UMMA K-major layout;
//   * one thread issues, per solve, the six products whose pieces reach
//     FP32 precision (x0 y0, x0 y1, x1 y0, x0 y2, x1 y1, x2 y0; the dropped
//     ones are below 2^-30 of the product) as tcgen05.mma kind::tf32
//     M=128 x N x K=8 into the solve's FP32 accumulator in tensor memory, and
//     commits them to the stage's mbarrier;
//   * two stages: the loads of step q+1 overlap the products of step q.
// Each product piece is exact in the FP32 accumulator (11 x 11 bits), so the
// rounding is that of FP32 accumulation, as in the SIMT rotation.  The tile's
// accumulators are read back with tcgen05.ld (lane = row) and written in the
// rotation's output layout.  Every mbarrier wait is bounded: on a timeout the
// CTA records an error flag, stops issuing work, waits (bounded) for its
// products in flight and frees its tensor memory.
#include <cstdint>

#include "bh_krylov.cuh"

namespace bh {

namespace {

constexpr int TC_M = 128;   // rows per tile = tensor-memory lanes
constexpr int TC_KS = 8;    // TF32 values per MMA K-step (32 bytes)
constexpr int TC_PIECES = 3;
constexpr unsigned TC_SPIN = 1u << 24;  // polls of an mbarrier before giving up
constexpr int TC_HEADER = 128;          // bytes of dynamic shared memory before the tiles

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of (row, k) in one K-step tile (K-major, no swizzle): core
// matrices of 8 rows x 16 bytes are contiguous; the two core matrices of a
// row group along K are 128 bytes apart, row groups 256 bytes apart.
__device__ __forceinline__ uint32_t tile_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor of a K-step tile at byte address addr.
__device__ __forceinline__ uint64_t tile_desc(uint32_t addr) {
    constexpr uint64_t lbo = 128 >> 4, sbo = 256 >> 4;
    return (uint64_t)((addr & 0x3FFFF) >> 4) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void split3(float x, float& a, float& b, float& c) {
    a = tf32_round(x);
    const float r1 = x - a;  // exact
    b = tf32_round(r1);
    c = tf32_round(r1 - b);  // exact difference, rounded to TF32
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned it = 0; it < TC_SPIN; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

// Shared memory (all dynamic, so that the launch may take the device's
// opt-in maximum): a 128-byte header (the two mbarriers, the tensor-memory
// address), B[g][piece][ks] tiles of npad rows (all K-steps of the CTA's
// coefficient matrices), then A[stage][g][piece] tiles of 128 rows.
__global__ void __launch_bounds__(128)
k_rotate_tc(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride,
            const float* __restrict__ V, const float* __restrict__ Yg, const int* __restrict__ in_idx,
            const int* __restrict__ out_idx, float* __restrict__ Vout, int64_t ostride, int ld_out,
            int single, int G, int npad, int nks, int tmem_cols, int64_t rows_per_cta,
            int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char s_tc[];
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_tc);
    uint32_t& s_tmem = *reinterpret_cast<uint32_t*>(s_tc + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int sg0 = blockIdx.x * G;
    const int nsg = min(G, Sproc - sg0);
    const size_t btile = (size_t)npad * 32, atile = (size_t)TC_M * 32;
    unsigned char* sB = s_tc + TC_HEADER;
    unsigned char* sA = sB + (size_t)G * TC_PIECES * nks * btile;
    const uint32_t bar0 = smem_u32(&s_bar[0]), bar1 = smem_u32(&s_bar[1]);

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1));
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // the coefficient matrices, split into TF32 pieces (zero beyond kc, nout)
    const int kcp = nks * TC_KS;
    for (int e = tid; e < G * kcp * npad; e += blockDim.x) {
        const int g = e / (kcp * npad), rem = e - g * (kcp * npad);
        const int c = rem / npad, o = rem - c * npad;
        const float y = (g < nsg && c < kc && o < nout) ? Yg[((size_t)(sg0 + g) * kc + c) * nout + o] : 0.f;
        float y0, y1, y2;
        split3(y, y0, y1, y2);
        const uint32_t off = tile_off(o, c & 7);
        unsigned char* base = sB + ((size_t)(g * TC_PIECES) * nks + c / TC_KS) * btile + off;
        *reinterpret_cast<float*>(base) = y0;
        *reinterpret_cast<float*>(base + (size_t)nks * btile) = y1;
        *reinterpret_cast<float*>(base + (size_t)2 * nks * btile) = y2;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(npad >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);
    int sin[4], sout[4];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        sin[g] = g < nsg ? in_idx[sg0 + g] : 0;
        sout[g] = g < nsg ? out_idx[sg0 + g] : 0;
    }

    const int64_t r0 = (int64_t)blockIdx.y * rows_per_cta;
    const int64_t r1 = min(D, r0 + rows_per_cta);
    const int64_t nstep = r1 > r0 ? (r1 - r0 + TC_M - 1) / TC_M * nks : 0;
    // the values of one K-step of this thread's row, loaded one step ahead so
    // that their latency overlaps the current step's stores and products
    float xr[4][TC_KS];
    auto load_step = [&](int64_t step) {
        const int64_t t0 = r0 + (step / nks) * TC_M;
        const int ks = (int)(step % nks);
        const int64_t row = t0 + tid;
        const bool live = row < r1;
        const float* vrow = V + (live ? row : t0) * (int64_t)ld_in;
#pragma unroll
        for (int g = 0; g < 4; ++g)
#pragma unroll
            for (int kk = 0; kk < TC_KS; ++kk) {
                const int c = ks * TC_KS + kk;
                xr[g][kk] = (g < nsg && live && c < kc)
                                ? vrow[(int64_t)(c / p) * bstride + (int64_t)sin[g] * p + c % p]
                                : 0.f;
            }
    };
    if (nstep > 0) load_step(0);
    uint32_t q = 0;  // K-steps whose products were committed
    bool ok = true;
    for (int64_t step = 0; step < nstep; ++step) {
        const int ks = (int)(step % nks);
        const int stage = (int)(step & 1);
        const uint32_t bar = stage ? bar1 : bar0;
        // the products of step - 2 read this stage: wait for them (every
        // thread polls; the CTA goes on only if all saw the arrival)
        if (step >= 2 && !__syncthreads_and(mbar_wait(bar, (uint32_t)((step - 2) >> 1) & 1) ? 1 : 0)) {
            ok = false;
            break;
        }
        unsigned char* aS = sA + (size_t)stage * G * TC_PIECES * atile;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            if (g >= G) break;
            unsigned char* ab = aS + (size_t)g * TC_PIECES * atile;
#pragma unroll
            for (int kk = 0; kk < TC_KS; ++kk) {
                float x0, x1, x2;
                split3(xr[g][kk], x0, x1, x2);
                const uint32_t off = tile_off(tid, kk);
                *reinterpret_cast<float*>(ab + off) = x0;
                *reinterpret_cast<float*>(ab + atile + off) = x1;
                *reinterpret_cast<float*>(ab + 2 * atile + off) = x2;
            }
        }
        if (step + 1 < nstep) load_step(step + 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int g = 0; g < nsg; ++g) {
                const uint32_t a0 = smem_u32(aS + (size_t)g * TC_PIECES * atile);
                const uint32_t b0 = smem_u32(sB + ((size_t)(g * TC_PIECES) * nks + ks) * btile);
                const uint32_t bstep = (uint32_t)(nks * btile), astep = (uint32_t)atile;
                const uint32_t d = tmem + (uint32_t)(g * npad);
                // (A piece, B piece): x0 y0, x0 y1, x1 y0, x0 y2, x1 y1, x2 y0
                mma_tf32(d, tile_desc(a0), tile_desc(b0), idesc, ks > 0 ? 1u : 0u);
                mma_tf32(d, tile_desc(a0), tile_desc(b0 + bstep), idesc, 1u);
                mma_tf32(d, tile_desc(a0 + astep), tile_desc(b0), idesc, 1u);
                mma_tf32(d, tile_desc(a0), tile_desc(b0 + 2 * bstep), idesc, 1u);
                mma_tf32(d, tile_desc(a0 + astep), tile_desc(b0 + bstep), idesc, 1u);
                mma_tf32(d, tile_desc(a0 + 2 * astep), tile_desc(b0), idesc, 1u);
            }
            mma_commit(bar);
        }
        q = (uint32_t)step + 1;
        if (ks != nks - 1) continue;
        // end of a tile: its products are complete once this step's commit arrives
        if (!__syncthreads_and(mbar_wait(bar, (uint32_t)(step >> 1) & 1) ? 1 : 0)) {
            ok = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int64_t row = r0 + (step / nks) * TC_M + tid;
        const bool live = row < r1;
        for (int g = 0; g < nsg; ++g) {
            for (int c0 = 0; c0 < npad; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(g * npad + c0), v);
                if (!live) continue;
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    const int i = c0 + u;
                    if (i >= nout) break;
                    if (single)
                        Vout[row * ld_out + (int64_t)sout[g] * nout + i] = v[u];
                    else
                        Vout[(int64_t)(i / p) * ostride + row * ld_out + (int64_t)sout[g] * p + i % p] = v[u];
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // every lane read before the next tile's first product overwrites
    }
    // ok is the same in every thread (all its changes follow __syncthreads_and)
    if (!ok && tid == 0 && status) atomicExch(status, 1);
    if (!ok && q > 0) {
        // products still in flight: wait (bounded) for the last commit
        const uint32_t ql = q - 1;
        (void)mbar_wait((ql & 1) ? bar1 : bar0, (ql >> 1) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
}

bool rotate_tc(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride, const float* V,
               const float* Yg, const int* in_idx, const int* out_idx, float* Vout, int64_t ostride,
               int ld_out, int single, int* d_status, cudaStream_t st) {
    if (Sproc <= 0 || D <= 0) return true;
    const int npad = (nout + 15) / 16 * 16;
    if (npad > 256 || kc <= 0 || p < 1 || p > 4) return false;
    const int nks = (kc + TC_KS - 1) / TC_KS;
    int G = std::max(1, std::min(Sproc, 4 / p));
    int smax = 0, dev = 0;
    BH_CUDA(cudaGetDevice(&dev));
    BH_CUDA(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    auto smem_of = [&](int g) {
        return (size_t)TC_HEADER + (size_t)g * TC_PIECES * nks * npad * 32 + (size_t)2 * g * TC_PIECES * TC_M * 32;
    };
    while (G > 1 && smem_of(G) > (size_t)smax) G /= 2;
    size_t smem = smem_of(G);
    if (smem > (size_t)smax) return false;
    int cols = 32;
    while (cols < G * npad) cols <<= 1;
    if (cols > 512) return false;
    // at most 512 / cols CTAs per SM hold tensor memory at once: request enough
    // shared memory that no more are resident
    const int per_sm_tmem = 512 / cols;
    const size_t sm_smem = 228 * 1024;
    const size_t min_smem = sm_smem / (per_sm_tmem + 1) + 1024;
    if (smem < min_smem && min_smem <= (size_t)smax) smem = min_smem;
    const int ngroups = (Sproc + G - 1) / G;
    const int64_t tiles = (D + TC_M - 1) / TC_M;
    const int per_sm = std::max(1, std::min(per_sm_tmem, (int)(sm_smem / (smem + 1024))));
    int64_t chunks = std::max<int64_t>(1, ((int64_t)2 * sm_count() * per_sm + ngroups - 1) / ngroups);
    chunks = std::min(chunks, tiles);
    const int64_t tiles_per = (tiles + chunks - 1) / chunks;
    chunks = (tiles + tiles_per - 1) / tiles_per;
    if (chunks > 65535) return false;
    allow_large_smem(k_rotate_tc, smem);
    k_rotate_tc<<<dim3((unsigned)ngroups, (unsigned)chunks), 128, smem, st>>>(
        D, Sproc, ld_in, p, kc, nout, bstride, V, Yg, in_idx, out_idx, Vout, ostride, ld_out, single, G, npad,
        nks, cols, tiles_per * TC_M, d_status);
    BH_CUDA(cudaGetLastError());
    return true;
}

}  // namespace bh
