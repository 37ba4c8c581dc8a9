// bh_noalloc.cu -- an allocation-free way to apply a built Hamiltonian.
//
// bh_hamiltonian_apply_noalloc computes y = H x like bh_hamiltonian_apply, but
// takes device pointers and a stream from the caller and performs no device
// or host allocation: no cudaMalloc/cudaFree, no stream or event creation, no
// allocating library call.  It is for callers that cannot allocate while they
// run -- for instance a solver loop inside a host application whose device
// memory is handed out once by its own pool, or many host threads driving one
// GPU, where cudaMalloc/cudaFree serialise against all other work on the
// device and a free-time synchronisation would stall the other threads.
//
// Its working memory (the solve parameters and, in the reference order, the
// two permuted vectors) lives in the file-scope device array below, which every
// GPU that loads this library holds until the process exits.  The host cannot
// use the array's name as a device address: at the first call on each device
// (with that device current) the address is looked up with
// cudaGetSymbolAddress and cached per device; that first call should therefore
// come before any stream capture.  All calls share the array and it keeps the
// contents of the last call; every word a call reads is written by the same
// call first (nothing needs to start at zero).  Calls that overlap on the GPU
// (different streams, or several host threads) race on the array and must be
// serialised by the caller.  The cached address belongs to the device's
// current context: after a cudaDeviceReset the process must not call this
// entry point again on that device.  In the lexicographic order the product
// reads x while it writes y, so x and y must not overlap (checked).
#include <mutex>

#include "bh_internal.h"
#include "bh_krylov.cuh"

namespace bh {

// 4 Mi doubles = 32 MiB: parameters (32 words) + 2 D nvec for the reference order
constexpr int64_t kApplyScratchDoubles = int64_t(4) << 20;
constexpr int64_t kApplyParamWords = 32;

static __device__ __align__(256) double g_apply_scratch[kApplyScratchDoubles];

__global__ void k_set_params(double* __restrict__ prm, double J, double U, double shift) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        prm[0] = J;
        prm[1] = U;
        prm[2] = shift;
    }
}

static double* apply_scratch_address() {
    static std::mutex mu;
    static double* addr[256] = {};
    int dev = 0;
    BH_CUDA(cudaGetDevice(&dev));
    BH_REQUIRE(dev >= 0 && dev < 256, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_apply_scratch);
        if (e != cudaSuccess || !p)
            throw Error(BH_ERR_CUDA, std::string("cudaGetSymbolAddress of the apply scratch failed: ") +
                                         cudaGetErrorString(e));
        addr[dev] = static_cast<double*>(p);
    }
    return addr[dev];
}

}  // namespace bh

extern "C" int bh_hamiltonian_apply_noalloc(const bh_hamiltonian* h, int order, double J, double U,
                                            double mu, int nvec, const double* x, double* y,
                                            void* stream) {
    try {
        BH_REQUIRE(h != nullptr && x != nullptr && y != nullptr, "null argument");
        BH_REQUIRE(nvec >= 1, "nvec must be >= 1");
        BH_REQUIRE(order == BH_ORDER_REFERENCE || order == BH_ORDER_LEX, "unknown order");
        const int64_t D = h->D;
        const int64_t need = bh::kApplyParamWords + (order == BH_ORDER_REFERENCE ? 2 * D * (int64_t)nvec : 0);
        if (need > bh::kApplyScratchDoubles)
            throw bh::Error(BH_ERR_ARG, "bh_hamiltonian_apply_noalloc: 2 * D * nvec = " +
                                            std::to_string(2 * D * (int64_t)nvec) +
                                            " doubles exceeds the fixed scratch of " +
                                            std::to_string(bh::kApplyScratchDoubles - bh::kApplyParamWords) +
                                            " doubles (32 MiB); use bh_hamiltonian_apply or fewer vectors");
        if (order == BH_ORDER_LEX) {
            // the product gathers rows of x while it writes y
            const uintptr_t n = (uintptr_t)(D * (int64_t)nvec) * sizeof(double);
            const uintptr_t xa = reinterpret_cast<uintptr_t>(x), ya = reinterpret_cast<uintptr_t>(y);
            BH_REQUIRE(xa + n <= ya || ya + n <= xa,
                       "bh_hamiltonian_apply_noalloc: x and y overlap (not allowed in the lexicographic order)");
        }
        int dev = 0;
        BH_CUDA(cudaGetDevice(&dev));
        BH_REQUIRE(dev == h->device, "the current device is not the Hamiltonian's device");
        double* s = bh::apply_scratch_address();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const bh::OpView<double> op = bh::op_view<double>(h);
        double* prm = s;
        bh::k_set_params<<<1, 32, 0, st>>>(prm, J, U, -mu * (double)h->n);
        BH_CUDA(cudaGetLastError());
        if (order == BH_ORDER_REFERENCE) {
            double* xl = s + bh::kApplyParamWords;
            double* yl = xl + D * (int64_t)nvec;
            bh::gather_rows(D, nvec, h->basis->d_col_of_lex.p, x, xl, st);
            bh::apply_operator_raw(op, nvec, nvec, prm, xl, yl, st);
            bh::gather_rows(D, nvec, h->basis->d_lex_of_col.p, yl, y, st);
        } else {
            bh::apply_operator_raw(op, nvec, nvec, prm, x, y, st);
        }
        BH_CUDA(cudaStreamSynchronize(st));
        bh::set_last_error("");
        return BH_OK;
    } catch (const bh::Error& e) {
        bh::set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        bh::set_last_error(e.what());
        return BH_ERR_ARG;
    }
}
