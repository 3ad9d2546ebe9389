// batch_kernels.cuh -- the persistent batched-stage kernel (batch.cu describes the scheme), shared by
// batch.cu (Cartesian instances) and batch_curv.cu (general geometry).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "flou_ctx.cuh"

namespace flou {

constexpr long long kWaitCycles = 200000000LL;   // per wait, ~0.1 s at 2 GHz

struct BatchArgs {
    const FaceParams* fp;        // [ninst], this stage
    const ElemParams* ep;        // [ninst], this stage
    const int32_t* inst_n;       // nodes per direction
    const int32_t* inst_lgl;     // basis with boundary nodes
    const int32_t* nface_items;  // face items per instance
    const int2* items;           // (instance | (G - 1) << 27 | kind << 30, first face node or element)
    int32_t nitems;
    int32_t ninst;
    int32_t* counter;            // [0] queue head, [1] abort flag, [2 + k] face items done of instance k
    int32_t* status;             // bit 0 non-physical, bit 1 wait timed out
    int32_t skip_done_inst;      // fault-injection hook: this instance never reports its faces (-1: none)
};

// One call per order, not inlined: each order's tile gets its own register allocation instead
// of the union of all orders (which would limit the persistent kernel to one block per SM).
// G consecutive tiles of EPB elements each (the last ones may run past the instance's elements).
template <int DIM, int N, int EQ, int VOL, int TP, int TB, bool CURV = false>
__device__ __noinline__ void batch_tile_n(const ElemParams& P, int lgl, int e0, int G, double* smem) {
    constexpr int EPB = Shape<DIM, N, TB>::EPB;
    for (int g = 0; g < G; ++g) {
        const int e = e0 + g * EPB;
        if (e >= P.nelem) break;   // uniform over the block
        if (g > 0) __syncthreads();   // the previous tile's last phase may still read shared memory
        if (VOL == FLOU_OP_STRONG) {
            if (lgl) strong_tile<DIM, N, EQ, true, TB, CURV>(P, e, smem);
            else strong_tile<DIM, N, EQ, false, TB, CURV>(P, e, smem);
        } else {
            split_tile<DIM, N, EQ, TP, true, TB, CURV>(P, e, smem);
        }
    }
}

template <int DIM, int EQ, bool CURV = false>
__device__ __noinline__ void batch_face(const FaceParams& P, int64_t gid, int lgl) {
    if (lgl) face_node<DIM, EQ, true, CURV>(P, gid);
    else face_node<DIM, EQ, false, CURV>(P, gid);
}

template <int DIM, int EQ, int VOL, int TP, int TB, bool CURV = false>
__device__ __forceinline__ void batch_tile(const ElemParams& P, int n, int lgl, int e0, int G, double* smem) {
    switch (n) {
        case 2: batch_tile_n<DIM, 2, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        case 3: batch_tile_n<DIM, 3, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        case 4: batch_tile_n<DIM, 4, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        case 5: batch_tile_n<DIM, 5, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        case 6: batch_tile_n<DIM, 6, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        case 7: batch_tile_n<DIM, 7, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
        default: batch_tile_n<DIM, 8, EQ, VOL, TP, TB, CURV>(P, lgl, e0, G, smem); break;
    }
}

template <int DIM, int EQ, int VOL, int TP, int TB, bool CURV = false>
__global__ void __launch_bounds__(TB, (TB >= 512 ? 1 : 1024 / TB)) batch_stage_kernel(BatchArgs A) {
    extern __shared__ double smem[];
    __shared__ int s_item;
    int32_t* done = A.counter + 2;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= A.nitems) break;
        const int2 w = A.items[it];
        const int inst = w.x & 0x07ffffff;
        if (!index_ok(inst, A.ninst, A.status, 0)) continue;
        if ((w.x >> 30) == 0) {
            const FaceParams& fp = A.fp[inst];
            const int64_t gid = (int64_t)w.y + threadIdx.x;
            batch_face<DIM, EQ, CURV>(fp, gid, A.inst_lgl[inst]);
            __threadfence();   // this thread's face fluxes are visible device-wide ...
            __syncthreads();   // ... for every thread of the block before the count goes up
            if (threadIdx.x == 0 && inst != A.skip_done_inst) atomicAdd(done + inst, 1);
        } else {
            if (threadIdx.x == 0) {
                const volatile int32_t* d = done + inst;
                const volatile int32_t* abort_flag = A.counter + 1;
                const int32_t target = A.nface_items[inst];
                const long long t0 = clock64();
                while (*d < target) {
                    if (*abort_flag) break;
                    if (clock64() - t0 > kWaitCycles) {
                        atomicExch(A.counter + 1, 1);
                        atomicOr(A.status, 2);
                        break;
                    }
                    __nanosleep(64);
                }
                __threadfence();
            }
            __syncthreads();
            batch_tile<DIM, EQ, VOL, TP, TB, CURV>(A.ep[inst], A.inst_n[inst], A.inst_lgl[inst], w.y,
                                             ((w.x >> 27) & 7) + 1, smem);
        }
    }
}

template <int DIM, int EQ, int VOL, int TP, int TB, bool CURV = false>
constexpr size_t batch_smem_bytes() {
    size_t m = 0;
    m = std::max(m, elem_smem_bytes<DIM, 2, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 3, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 4, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 5, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 6, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 7, EQ, VOL, TP, TB, CURV>());
    m = std::max(m, elem_smem_bytes<DIM, 8, EQ, VOL, TP, TB, CURV>());
    return (m + 15) & ~size_t(15);
}

// The instantiated batch kernels: 2D Euler strong form (the batched configuration) with 128 or
// 256 threads per block, 3D Euler split form with the Chandrashekar flux with 512.
struct BatchKernel {
    int dim, eq, vol, tp, tb;
    bool curv;   // general geometry (every instance of the batch)
    void (*fn)(BatchArgs);
    size_t smem;
};

// The general-geometry batch kernels (batch_curv.cu): the same list for curvilinear instances.
extern const BatchKernel kBatchKernelsCurv[];
extern const int kNumBatchKernelsCurv;

}  // namespace flou
