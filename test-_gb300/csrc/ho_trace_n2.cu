// Instantiation of the trace kernel for 2 modes per direction.
#include "ho_trace.cuh"

namespace ho {
template cudaError_t launch_n<2>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
}  // namespace ho
