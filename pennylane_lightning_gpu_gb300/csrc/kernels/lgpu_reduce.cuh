// Deterministic FP64 reductions: each block folds its items in a fixed order,
// writes one partial, and the last block to arrive sums the partials in block
// order.  The grid size is a fixed multiple of the SM count, so a given state
// on a given GPU always produces the same bits.
#pragma once

#include "lgpu_internal.cuh"

namespace lgpu {

constexpr int kReduceBlock = 256;

inline unsigned reduce_grid(uint64_t items) {
    return grid_for(items, kReduceBlock, 8, 4);
}

// Scratch layout for single-value reductions: [counter(256 B)][partials ...]
struct ReduceScratch {
    unsigned *counter;
    double2 *partials;
};
lgpu_status_t reduce_scratch(lgpu_context_t ctx, unsigned grid, unsigned nout, ReduceScratch *rs);

// Body: __device__ double2 operator()(I item) const
template <int NOUT, class I, class Body>
__global__ void __launch_bounds__(kReduceBlock)
    reduce_kernel(Body body, I nitems, double2 *partials, unsigned *counter, double2 *out) {
    __shared__ double2 sm[kReduceBlock / 32];
    double2 acc[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) acc[k] = make_double2(0.0, 0.0);
    const I stride = I(gridDim.x) * kReduceBlock;
    for (I i = I(blockIdx.x) * kReduceBlock + threadIdx.x; i < nitems; i += stride) {
        body(i, acc);
    }
#pragma unroll
    for (int k = 0; k < NOUT; k++) {
        double2 v = block_reduce_d2<kReduceBlock>(acc[k], sm);
        if (threadIdx.x == 0) partials[size_t(blockIdx.x) * NOUT + k] = v;
        __syncthreads();
    }
    if (last_block_arrive(counter)) {
#pragma unroll
        for (int k = 0; k < NOUT; k++) {
            double2 s = make_double2(0.0, 0.0);
            for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
                const double2 p = __ldcg(&partials[size_t(b) * NOUT + k]);
                s.x += p.x;
                s.y += p.y;
            }
            s = block_reduce_d2<kReduceBlock>(s, sm);
            if (threadIdx.x == 0) out[k] = s;
            __syncthreads();
        }
        if (threadIdx.x == 0) *counter = 0u;
    }
}

// Copy `count` double2 results from device `src` to the caller's `out`
// (host or device) and synchronise when the destination is host memory.
lgpu_status_t deliver(lgpu_context_t ctx, const double2 *src, size_t count, double *out,
                      int out_on_device, cudaStream_t s);

}  // namespace lgpu
