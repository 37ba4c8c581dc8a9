// bh_dense.cu -- dense symmetric eigensolver on the device.
//
// Replaces Op::exact_eigen (src/operator.cpp:92-101), which converts the
// sparse matrix to a dense Eigen matrix and calls SelfAdjointEigenSolver.  The
// dense problem only exists for small sectors; it is handed to cuSOLVER's
// divide-and-conquer syevd (a library call, like a cuBLAS GEMM).
#include <cusolverDn.h>

#include "bh_internal.h"

namespace bh {

void dense_eigh(int64_t n, const double* h_a, double* h_w, double* h_z) {
    BH_REQUIRE(n >= 1 && n <= 32768, "dense eigensolve limited to n <= 32768");
    Stream st;
    cusolverDnHandle_t hs = nullptr;
    if (cusolverDnCreate(&hs) != CUSOLVER_STATUS_SUCCESS) throw Error(BH_ERR_CUDA, "cusolverDnCreate failed");
    struct Guard {
        cusolverDnHandle_t h;
        ~Guard() { cusolverDnDestroy(h); }
    } guard{hs};
    cusolverDnSetStream(hs, st);
    DevBuf<double> a((size_t)n * n), w(n);
    DevBuf<int> info(1);
    BH_CUDA(cudaMemcpyAsync(a.p, h_a, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, st));
    int lwork = 0;
    const cublasFillMode_t up = CUBLAS_FILL_MODE_UPPER;
    const cusolverEigMode_t mode = h_z ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
    if (cusolverDnDsyevd_bufferSize(hs, mode, up, (int)n, a.p, (int)n, w.p, &lwork) != CUSOLVER_STATUS_SUCCESS)
        throw Error(BH_ERR_CUDA, "cusolverDnDsyevd_bufferSize failed");
    DevBuf<double> work((size_t)std::max(lwork, 1));
    if (cusolverDnDsyevd(hs, mode, up, (int)n, a.p, (int)n, w.p, work.p, lwork, info.p) != CUSOLVER_STATUS_SUCCESS)
        throw Error(BH_ERR_CUDA, "cusolverDnDsyevd failed");
    int hinfo = 0;
    BH_CUDA(cudaMemcpyAsync(&hinfo, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaMemcpyAsync(h_w, w.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (h_z) BH_CUDA(cudaMemcpyAsync(h_z, a.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
    if (hinfo != 0) throw Error(BH_ERR_NOCONV, "Eigenvalue computation failed.");
}

}  // namespace bh
