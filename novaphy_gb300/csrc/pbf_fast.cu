// Fast build of the PBF kernels: FMA contraction and rsqrt in the spiky
// gradient; same summation order as the exact build.
#define PBF_FAST 1
#define PBF_NS fast
#include "pbf_kernels.cuh"
#include "pbf_launch.cuh"

namespace pbf {

cudaError_t fast_enqueue_step(const StepBuffers& B, const StepConsts& C, int iters,
                               SortScratch& sort, cudaStream_t st, PhaseMarks* pm,
                               const BoundaryGrid* bg) {
    return fast::enqueue_step(B, C, iters, sort, st, pm, bg);
}

cudaError_t fast_enqueue_batch(const StepBuffers& B, const BatchDesc& D, SortScratch& sort,
                                cudaStream_t st, PhaseMarks* pm) {
    return fast::enqueue_batch_step(B, D, sort, st, pm);
}

int fast_persist_blocks() { return fast::persist_blocks_max(); }

}  // namespace pbf
