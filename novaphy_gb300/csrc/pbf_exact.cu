// Exact-arithmetic build of the PBF kernels: compiled with -fmad=false and
// IEEE division / square root, so results round like the reference's float
// code operation by operation.
#define PBF_FAST 0
#define PBF_NS exact
#include "pbf_kernels.cuh"
#include "pbf_launch.cuh"

namespace pbf {

cudaError_t exact_enqueue_step(const StepBuffers& B, const StepConsts& C, int iters,
                               SortScratch& sort, cudaStream_t st, PhaseMarks* pm,
                               const BoundaryGrid* bg) {
    return exact::enqueue_step(B, C, iters, sort, st, pm, bg);
}

cudaError_t exact_enqueue_batch(const StepBuffers& B, const BatchDesc& D, SortScratch& sort,
                                cudaStream_t st, PhaseMarks* pm) {
    return exact::enqueue_batch_step(B, D, sort, st, pm);
}

int exact_persist_blocks() { return exact::persist_blocks_max(); }

cudaError_t debug_cells(const StepBuffers& B, const StepConsts& C, int* d_cells3,
                        cudaStream_t st) {
    if (C.n <= 0) return cudaSuccess;
    exact::k_debug_cells<<<exact::grid_of(C.n, exact::kBlock), exact::kBlock, 0, st>>>(
        B.x, B.v, d_cells3, C);
    return cudaGetLastError();
}

cudaError_t debug_neighbors(const StepBuffers& B, const StepConsts& C, SortScratch& sort,
                            long long* d_cnt, const long long* d_offs, int* d_out, long long cap,
                            int fill, cudaStream_t st) {
    if (C.n <= 0) return cudaSuccess;
    if (!fill) {
        cudaError_t e = exact::enqueue_prefix(B, C, sort, st);
        if (e != cudaSuccess) return e;
    }
    exact::k_debug_neighbors<<<exact::grid_of(C.n, exact::kBlock), exact::kBlock, 0, st>>>(
        B.xa, B.sx, d_cnt, d_offs, d_out, cap, fill, exact::grid_view(B), C);
    return cudaGetLastError();
}

}  // namespace pbf
