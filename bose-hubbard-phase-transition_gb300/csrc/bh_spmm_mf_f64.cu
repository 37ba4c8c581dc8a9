// bh_spmm_mf_f64.cu -- the matrix-free Y = H X kernels for double vectors (see
// bh_spmm.cuh); one translation unit per (operator kind, type) so they build in parallel.
#include "bh_spmm.cuh"

namespace bh {
template double launch_spmm_kind<double, true>(const OpView<double>&, int, int, const double*, const double*,
                                          double*, cudaStream_t, double*, int*, bool);
template double launch_spmm_shape_kind<double, true>(const OpView<double>&, int, int, const double*,
                                                const double*, double*, cudaStream_t, const SpmmShape&);
template int tune_spmm_kind<double, true>(const OpView<double>&, int, int, const double*, const double*, double*,
                                     cudaStream_t, bool, bool, TuneEntry*);
}  // namespace bh
