// Entry points of the two kernel builds (pbf_exact.cu, pbf_fast.cu).
#pragma once

#include "pbf_types.cuh"
#include "radix_sort.cuh"

namespace pbf {

// bg: the Akinci boundary of a two-way coupled step, else null.
cudaError_t exact_enqueue_step(const StepBuffers& B, const StepConsts& C, int iters,
                               SortScratch& sort, cudaStream_t st, PhaseMarks* pm = nullptr,
                               const BoundaryGrid* bg = nullptr);
cudaError_t fast_enqueue_step(const StepBuffers& B, const StepConsts& C, int iters,
                              SortScratch& sort, cudaStream_t st, PhaseMarks* pm = nullptr,
                              const BoundaryGrid* bg = nullptr);

// One step of a batch of scenes (B holds the batch's scratch; the scenes'
// state is reached through D.refs).
cudaError_t exact_enqueue_batch(const StepBuffers& B, const BatchDesc& D, SortScratch& sort,
                                cudaStream_t st, PhaseMarks* pm = nullptr);
cudaError_t fast_enqueue_batch(const StepBuffers& B, const BatchDesc& D, SortScratch& sort,
                               cudaStream_t st, PhaseMarks* pm = nullptr);
// Largest co-resident grid of the persistent Jacobi loop on the current device.
int exact_persist_blocks();
int fast_persist_blocks();

// Parity probes (exact build).
cudaError_t debug_cells(const StepBuffers& B, const StepConsts& C, int* d_cells3,
                        cudaStream_t st);
cudaError_t debug_neighbors(const StepBuffers& B, const StepConsts& C, SortScratch& sort,
                            long long* d_cnt, const long long* d_offs, int* d_out, long long cap,
                            int fill, cudaStream_t st);

}  // namespace pbf
