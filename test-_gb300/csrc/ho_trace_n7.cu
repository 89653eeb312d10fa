// Instantiations of the trace kernels for 7 modes per direction.
#include "ho_check.cuh"
#include "ho_rounds.cuh"
#include "ho_trace.cuh"

namespace ho {
template cudaError_t launch_n<7>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
template cudaError_t launch_round_n<7>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
template cudaError_t launch_residuals_n<7>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                           double*, cudaStream_t);
template cudaError_t launch_tail_n<7>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*, bool,
                                      cudaStream_t);
template cudaError_t launch_check_n<7>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, uint32_t*,
                                         unsigned*, unsigned*, int64_t, int, cudaStream_t);
}  // namespace ho
