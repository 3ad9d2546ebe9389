// batch.cu -- many independent discretizations (uneven element counts and orders) advanced
// together: one persistent launch per stage (SSP-RK3's three, or the instances' common
// 2N-storage method's) serves every instance from one work queue, and the stages of a step are
// replayed as one CUDA graph; an instance with the Zhang-Shu limiter gets it after every stage
// and one with monitors records them after every step (its own launches in the graph).  A batch
// is all Cartesian or all on general geometry (batch_curv.cu instantiates the latter).
//
// Work queue of one stage: first every face item of every instance (TB face nodes each), then
// every element item (G consecutive element tiles of the instance's order, G chosen per order by
// the autotuner).  Blocks take items with an
// atomic counter.  An element item needs the face fluxes of its instance; because all face
// items precede all element items in the queue, they have all been taken by running blocks
// when an element item is taken, so the wait below always ends.  It is still bounded: after
// ~0.1 s it raises FLOU_ERR_TIMEOUT through the status word and an abort flag that stops all
// later waits, instead of hanging the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch_kernels.cuh"

namespace flou {

static const BatchKernel kBatchKernels[] = {
    {2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128, false,
     batch_stage_kernel<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128>,
     batch_smem_bytes<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 128>()},
    {2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256, false,
     batch_stage_kernel<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256>,
     batch_smem_bytes<2, FLOU_EQ_EULER, FLOU_OP_STRONG, FLOU_TP_STD_AVERAGE, 256>()},
    {3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512, false,
     batch_stage_kernel<3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512>,
     batch_smem_bytes<3, FLOU_EQ_EULER, FLOU_OP_SPLIT, FLOU_TP_CHANDRASHEKAR, 512>()},
};

}  // namespace flou

using namespace flou;

struct flou_batch {
    int n = 0;
    std::vector<flou_ctx*> ctxs;
    int dim = 0, eq = 0, vol = 0, tp = 0;
    std::string err;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    std::vector<const BatchKernel*> kernels;   // candidates for this batch's equation/operator
    const BatchKernel* kern = nullptr;
    int blocks_per_sm = 0, order = 0, sms = 0;
    int tiles[MAXN + 1] = {};   // element tiles per work item for n nodes per direction (0: one)
    // stages of a step: SSP-RK3's three, or the instances' common 2N-storage method; the
    // parameter sets hold one per stage and instance, then a timing set (the first SSP-RK3 stage,
    // which writes only the stage buffer) for the autotuner
    int nst = 3;
    bool any_limiter = false, any_monitors = false;
    std::vector<double*> Q;
    std::vector<double> dt;
    bool have_states = false;
    FaceParams* d_fp = nullptr;
    ElemParams* d_ep = nullptr;
    int32_t* d_meta = nullptr;   // inst_n[n], inst_lgl[n], nface_items[n]
    int2* d_items = nullptr;
    int nitems = 0;
    int32_t* d_counter = nullptr;
    int32_t* d_status = nullptr;
    int skip_done_inst = -1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
};

namespace {

int bfail(flou_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

int bcuda(flou_batch* b, cudaError_t e, const char* what) {
    return bfail(b, e == cudaErrorMemoryAllocation ? FLOU_ERR_OOM : FLOU_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

#define BCK(call, what)                                  \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return bcuda(b, _e, what); \
    } while (0)

void drop_graph(flou_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
}

int epb_of(int npe, int tb) { return npe >= tb ? 1 : tb / npe; }

// Queue of one stage: all face items (instance order), then all element items (instance order,
// or orders descending when `order` is 1 -- the largest tiles first).
int build_items(flou_batch* b) {
    int tb = b->kern->tb;
    std::vector<int2> items;
    std::vector<int32_t> meta(3 * b->n);
    for (int k = 0; k < b->n; ++k) {
        flou_ctx* c = b->ctxs[k];
        int64_t fn = c->nfdofs;
        int nfi = (int)((fn + tb - 1) / tb);
        for (int j = 0; j < nfi; ++j) items.push_back(make_int2(k, j * tb));
        meta[k] = c->n;
        meta[b->n + k] = c->lgl ? 1 : 0;
        meta[2 * b->n + k] = nfi;
    }
    std::vector<int> korder(b->n);
    for (int k = 0; k < b->n; ++k) korder[k] = k;
    if (b->order == 1)
        std::stable_sort(korder.begin(), korder.end(), [&](int x, int y) { return b->ctxs[x]->n > b->ctxs[y]->n; });
    for (int k : korder) {
        flou_ctx* c = b->ctxs[k];
        int epb = epb_of(c->npe, b->kern->tb);
        int G = std::max(1, std::min(8, b->tiles[c->n]));
        for (int e = 0; e < c->nelem; e += epb * G) items.push_back(make_int2(k | ((G - 1) << 27) | (1 << 30), e));
    }
    if (items.size() > 0x7fffffff) return bfail(b, FLOU_ERR_ARG, "too many work items");
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    BCK(cudaMalloc((void**)&b->d_items, items.size() * sizeof(int2)), "item table");
    BCK(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice), "item table");
    BCK(cudaMemcpy(b->d_meta, meta.data(), meta.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "instance table");
    b->nitems = (int)items.size();
    return FLOU_OK;
}

int upload_params(flou_batch* b) {
    const int ns = b->nst;
    std::vector<FaceParams> fp((ns + 1) * b->n);
    std::vector<ElemParams> ep((ns + 1) * b->n);
    for (int k = 0; k < b->n; ++k) {
        flou_ctx* c = b->ctxs[k];
        double* Q = b->Q[k];
        double* U = c->d_U;
        double dt = b->dt[k];
        if (c->lsrk_s) {   // 2N-storage: every stage in place on Q, the register in U
            for (int st = 0; st < ns; ++st) {
                fp[st * b->n + k] = ctx_face_params(c, Q);
                ep[st * b->n + k] = ctx_elem_params(c, Q, U, Q, 3, dt, st ? c->lsrk_A[st] : 0.0, c->lsrk_B[st]);
            }
        } else {
            fp[k] = ctx_face_params(c, Q);
            fp[b->n + k] = ctx_face_params(c, U);
            fp[2 * b->n + k] = ctx_face_params(c, U);
            ep[k] = ctx_elem_params(c, Q, Q, U, 1, dt, 0.0, 1.0);
            ep[b->n + k] = ctx_elem_params(c, U, Q, U, 2, dt, 0.75, 0.25);
            ep[2 * b->n + k] = ctx_elem_params(c, U, Q, Q, 2, dt, 1.0 / 3.0, 2.0 / 3.0);
        }
        fp[ns * b->n + k] = ctx_face_params(c, Q);   // the timing set
        ep[ns * b->n + k] = ctx_elem_params(c, Q, Q, U, 1, dt, 0.0, 1.0);
        for (int s = 0; s <= ns; ++s) {
            ep[s * b->n + k].status = b->d_status;
            fp[s * b->n + k].status = b->d_status;
        }
    }
    BCK(cudaMemcpy(b->d_fp, fp.data(), fp.size() * sizeof(FaceParams), cudaMemcpyHostToDevice), "stage parameters");
    BCK(cudaMemcpy(b->d_ep, ep.data(), ep.size() * sizeof(ElemParams), cudaMemcpyHostToDevice), "stage parameters");
    return FLOU_OK;
}

int grid_of(flou_batch* b, int* grid) {
    int per_sm = b->blocks_per_sm;
    int maxb = 0;
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, b->kern->fn, b->kern->tb, b->kern->smem), "occupancy");
    if (maxb < 1) return bfail(b, FLOU_ERR_CUDA, "batch kernel cannot be resident");
    if (per_sm <= 0 || per_sm > maxb) per_sm = maxb;
    *grid = b->sms * per_sm;
    return FLOU_OK;
}

int launch_stage(flou_batch* b, int s, cudaStream_t st) {
    int grid = 0, r;
    if ((r = grid_of(b, &grid))) return r;
    BCK(cudaMemsetAsync(b->d_counter, 0, (2 + b->n) * sizeof(int32_t), st), "queue reset");
    BatchArgs A;
    A.fp = b->d_fp + s * b->n;
    A.ep = b->d_ep + s * b->n;
    A.inst_n = b->d_meta;
    A.inst_lgl = b->d_meta + b->n;
    A.nface_items = b->d_meta + 2 * b->n;
    A.items = b->d_items;
    A.nitems = b->nitems;
    A.ninst = b->n;
    A.counter = b->d_counter;
    A.status = b->d_status;
    A.skip_done_inst = b->skip_done_inst;
    b->kern->fn<<<grid, b->kern->tb, b->kern->smem, st>>>(A);
    BCK(cudaGetLastError(), "batch kernel launch");
    return FLOU_OK;
}

// The limiter after stage s of every instance that has one (OrdinaryDiffEq's stage_limiter!):
// on the stage buffer after the first two SSP-RK3 stages, on the state otherwise.
int limit_stage(flou_batch* b, int s, cudaStream_t st) {
    if (!b->any_limiter) return FLOU_OK;
    for (int k = 0; k < b->n; ++k) {
        flou_ctx* c = b->ctxs[k];
        if (!c->limiter) continue;
        double* q = (!c->lsrk_s && s < 2) ? c->d_U : b->Q[k];
        int r = ctx_limit(c, st, q);
        if (r) return bfail(b, r, "instance " + std::to_string(k) + ": " + c->err);
    }
    return FLOU_OK;
}

// The monitors of every instance that records them, after each step (Flou's monitor callback).
int record_monitors(flou_batch* b, cudaStream_t st) {
    if (!b->any_monitors) return FLOU_OK;
    for (int k = 0; k < b->n; ++k) {
        flou_ctx* c = b->ctxs[k];
        if (!c->mon_mask) continue;
        int r = ctx_record_monitors(c, st, b->Q[k]);
        if (r) return bfail(b, r, "instance " + std::to_string(k) + ": " + c->err);
    }
    return FLOU_OK;
}

int check_status(flou_batch* b) {
    int32_t st[2];
    BCK(cudaMemcpyAsync(st, b->d_status, sizeof(st), cudaMemcpyDeviceToHost, b->stream), "status read");
    BCK(cudaStreamSynchronize(b->stream), "stream synchronize");
    if (st[0]) {
        int32_t init[2] = {0, 0x7fffffff};
        cudaMemcpy(b->d_status, init, sizeof(init), cudaMemcpyHostToDevice);
        if (st[0] & 4)
            return bfail(b, FLOU_ERR_INDEX, "a device index check failed (element " + std::to_string(st[1]) +
                                                " of an instance; FLOU_CUDA_CHECKED build)");
        if (st[0] & 2) return bfail(b, FLOU_ERR_TIMEOUT, "a batched element tile waited too long for its face fluxes");
        return bfail(b, FLOU_ERR_NONPHYSICAL, "non-physical or non-finite state in element " + std::to_string(st[1]) +
                                                  " of an instance");
    }
    return FLOU_OK;
}

}  // namespace

extern "C" {

const char* flou_batch_last_error(const flou_batch* b) { return b ? b->err.c_str() : "null batch"; }

int32_t flou_batch_create(int32_t n, flou_ctx* const* ctxs, flou_batch** out) {
    if (!out || n <= 0 || n >= (1 << 27) || !ctxs) return FLOU_ERR_ARG;
    *out = nullptr;
    flou_batch* b = new flou_batch();
    b->n = n;
    b->ctxs.assign(ctxs, ctxs + n);
    flou_ctx* c0 = ctxs[0];
    if (!c0) { delete b; return FLOU_ERR_ARG; }
    b->dim = c0->cfg.dim;
    b->eq = c0->cfg.equation;
    b->vol = c0->cfg.volume_op;
    b->tp = b->vol == FLOU_OP_SPLIT ? c0->cfg.twopoint_flux : FLOU_TP_STD_AVERAGE;
    // Cartesian or general geometry: one kernel list or the other, for the whole batch
    const BatchKernel* list = c0->curv ? kBatchKernelsCurv : kBatchKernels;
    const int nlist = c0->curv ? kNumBatchKernelsCurv : (int)(sizeof(kBatchKernels) / sizeof(kBatchKernels[0]));
    for (int i = 0; i < nlist; ++i) {
        const BatchKernel& k = list[i];
        if (k.dim == b->dim && k.eq == b->eq && k.vol == b->vol && k.tp == b->tp) b->kernels.push_back(&k);
    }
    if (b->kernels.empty()) {
        delete b;
        return FLOU_ERR_UNSUPPORTED;
    }
    int maxnpe = 0;
    for (int k = 0; k < n; ++k) {
        flou_ctx* c = ctxs[k];
        if (!c || c->cfg.dim != b->dim || c->cfg.equation != b->eq || c->cfg.volume_op != b->vol ||
            (b->vol == FLOU_OP_SPLIT && c->cfg.twopoint_flux != b->tp)) {
            delete b;
            return FLOU_ERR_ARG;
        }
        int r = ctx_prepare(c);
        if (r) {
            delete b;
            return r;
        }
        if (c->cfg.volume_op != FLOU_OP_STRONG && !c->bnodes) {
            c->err = "the batched launch covers the split form on Gauss-Lobatto nodes";
            delete b;
            return FLOU_ERR_UNSUPPORTED;
        }
        if (c->curv != c0->curv) {
            c->err = "the instances of a batch are all on Cartesian or all on general geometry";
            delete b;
            return FLOU_ERR_ARG;
        }
        if (c->mon_mask) b->any_monitors = true;
        // one stage sequence for all: SSP-RK3 everywhere, or one 2N-storage method everywhere
        bool same = c->lsrk_s == c0->lsrk_s;
        for (int st = 0; same && st < c->lsrk_s; ++st)
            same = c->lsrk_A[st] == c0->lsrk_A[st] && c->lsrk_B[st] == c0->lsrk_B[st];
        if (!same) {
            c->err = "the instances of a batch step with the same time integrator";
            delete b;
            return FLOU_ERR_ARG;
        }
        if (c->limiter) b->any_limiter = true;
        maxnpe = std::max(maxnpe, c->npe);
    }
    std::vector<const BatchKernel*> fit;
    for (const BatchKernel* k : b->kernels)
        if (k->tb >= maxnpe) fit.push_back(k);
    if (fit.empty()) {
        delete b;
        return FLOU_ERR_UNSUPPORTED;
    }
    b->kernels = fit;
    b->kern = fit.back();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    b->nst = c0->lsrk_s ? c0->lsrk_s : 3;
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_fp, (size_t)(b->nst + 1) * n * sizeof(FaceParams));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_ep, (size_t)(b->nst + 1) * n * sizeof(ElemParams));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_meta, 3 * n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_counter, (2 + n) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_status, 2 * sizeof(int32_t));
    for (const BatchKernel* k : b->kernels)
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k->smem);
    if (e != cudaSuccess) {
        *out = b;   // let the caller read the message, then destroy
        b->err = std::string("batch set-up: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FLOU_ERR_OOM : FLOU_ERR_CUDA;
    }
    int32_t init[2] = {0, 0x7fffffff};
    cudaMemcpy(b->d_status, init, sizeof(init), cudaMemcpyHostToDevice);
    b->stream = b->own_stream;
    b->Q.assign(n, nullptr);
    b->dt.assign(n, 0.0);
    int r = build_items(b);
    *out = b;
    return r;
}

int32_t flou_batch_destroy(flou_batch* b) {
    if (!b) return FLOU_ERR_ARG;
    drop_graph(b);
    void* bufs[] = {b->d_fp, b->d_ep, b->d_meta, b->d_items, b->d_counter, b->d_status};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return FLOU_OK;
}

int32_t flou_batch_set_stream(flou_batch* b, void* stream) {
    if (!b) return FLOU_ERR_ARG;
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    return FLOU_OK;
}

int32_t flou_batch_set_states(flou_batch* b, double* const* Q, const double* dt) {
    if (!b || !Q || !dt) return FLOU_ERR_ARG;
    for (int k = 0; k < b->n; ++k) {
        if (!Q[k]) return bfail(b, FLOU_ERR_ARG, "null state of instance " + std::to_string(k));
        if (!std::isfinite(dt[k])) return bfail(b, FLOU_ERR_ARG, "non-finite dt of instance " + std::to_string(k));
        b->Q[k] = Q[k];
        b->dt[k] = dt[k];
    }
    int r = upload_params(b);
    if (r) return r;
    b->have_states = true;
    drop_graph(b);
    return FLOU_OK;
}

int32_t flou_batch_step(flou_batch* b, int32_t nsteps) {
    if (!b) return FLOU_ERR_ARG;
    if (!b->have_states) return bfail(b, FLOU_ERR_STATE, "flou_batch_set_states has not been called");
    if (nsteps < 0) return bfail(b, FLOU_ERR_ARG, "negative nsteps");
    if (nsteps == 0) return FLOU_OK;
    if (!b->gexec) {
        BCK(cudaStreamBeginCapture(b->own_stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        int rr = FLOU_OK;
        for (int s = 0; s < b->nst && !rr; ++s) {
            rr = launch_stage(b, s, b->own_stream);
            if (!rr) rr = limit_stage(b, s, b->own_stream);
        }
        if (!rr) rr = record_monitors(b, b->own_stream);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(b->own_stream, &g);
        if (rr) { if (g) cudaGraphDestroy(g); return rr; }
        if (ce != cudaSuccess) return bcuda(b, ce, "graph capture");
        b->graph = g;
        BCK(cudaGraphInstantiate(&b->gexec, g, 0), "graph instantiate");
    }
    for (int s = 0; s < nsteps; ++s) BCK(cudaGraphLaunch(b->gexec, b->stream), "graph launch");
    return check_status(b);
}

// Chooses the block size (elements per tile follow from it: tb / n^d per order), the resident
// blocks per SM and the element-item order by timing the first stage (which writes only the
// stage buffers) for every candidate, then, order by order, how many element tiles one work item
// holds (1, 2 or 4: larger items take fewer queue operations and face-count checks, smaller ones
// balance the tail), each against the timing of the current choice.  out = {threads per block,
// blocks per SM, order}; flou_batch_tiles reads the per-order tiles per item.
int32_t flou_batch_autotune(flou_batch* b, int32_t* out) {
    if (!b) return FLOU_ERR_ARG;
    if (!b->have_states) return bfail(b, FLOU_ERR_STATE, "flou_batch_set_states has not been called");
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0), "event");
    BCK(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    const BatchKernel* bk = b->kern;
    int bb = 0, bo = 0;
    for (const BatchKernel* k : b->kernels) {
        b->kern = k;
        int maxb = 0;
        BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, k->fn, k->tb, k->smem), "occupancy");
        for (int order = 0; order < 2; ++order) {
            b->order = order;
            int r = build_items(b);
            if (r) return r;
            for (int per = 1; per <= maxb; per *= 2) {
                b->blocks_per_sm = per;
                float tot = 0.f;
                for (int rep = 0; rep < 3; ++rep) {
                    BCK(cudaEventRecord(e0, b->stream), "event");
                    if ((r = launch_stage(b, b->nst, b->stream))) return r;
                    BCK(cudaEventRecord(e1, b->stream), "event");
                    BCK(cudaEventSynchronize(e1), "event");
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) tot += ms;
                }
                if (tot < best) { best = tot; bk = k; bb = per; bo = order; }
            }
        }
    }
    b->kern = bk;
    b->blocks_per_sm = bb;
    b->order = bo;
    // tiles per element item, one order at a time (coordinate search from one tile everywhere)
    auto time_stage = [&](float* ms_out) -> int {
        int r = build_items(b);
        if (r) return r;
        float tot = 0.f;
        for (int rep = 0; rep < 3; ++rep) {
            BCK(cudaEventRecord(e0, b->stream), "event");
            if ((r = launch_stage(b, b->nst, b->stream))) return r;
            BCK(cudaEventRecord(e1, b->stream), "event");
            BCK(cudaEventSynchronize(e1), "event");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) tot += ms;
        }
        *ms_out = tot;
        return FLOU_OK;
    };
    bool present[MAXN + 1] = {};
    for (flou_ctx* c : b->ctxs) present[c->n] = true;
    for (int n = 0; n <= MAXN; ++n) b->tiles[n] = 1;
    float cur = 0.f;
    int r = time_stage(&cur);
    if (r) return r;
    for (int n = 2; n <= MAXN; ++n) {
        if (!present[n]) continue;
        int bestG = b->tiles[n];
        for (int G : {2, 4}) {
            b->tiles[n] = G;
            float t = 0.f;
            if ((r = time_stage(&t))) return r;
            if (t < cur) { cur = t; bestG = G; }
        }
        b->tiles[n] = bestG;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    r = build_items(b);
    if (r) return r;
    drop_graph(b);
    if (out) { out[0] = bk->tb; out[1] = bb; out[2] = bo; }
    return check_status(b);
}

// Element tiles per work item for n = 2..MAXN nodes per direction (tiles[n - 2]; 1 before tuning).
int32_t flou_batch_tiles(const flou_batch* b, int32_t* tiles) {
    if (!b || !tiles) return FLOU_ERR_ARG;
    for (int n = 2; n <= MAXN; ++n) tiles[n - 2] = std::max(1, b->tiles[n]);
    return FLOU_OK;
}

// Sets the element tiles per work item of every order (1..8 each) instead of tuning them.
int32_t flou_batch_set_tiles(flou_batch* b, const int32_t* tiles) {
    if (!b || !tiles) return FLOU_ERR_ARG;
    for (int n = 2; n <= MAXN; ++n)
        if (tiles[n - 2] < 1 || tiles[n - 2] > 8)
            return bfail(b, FLOU_ERR_ARG, "tiles per work item must be 1..8 (order " + std::to_string(n - 1) + ")");
    for (int n = 2; n <= MAXN; ++n) b->tiles[n] = tiles[n - 2];
    int r = build_items(b);
    if (r) return r;
    drop_graph(b);
    return FLOU_OK;
}

// Fault-injection hook for tests: the face items of instance `inst` never report completion,
// so that instance's element tiles exhaust their bounded wait (-1 restores normal operation).
int32_t flou_batch_test_skip_faces(flou_batch* b, int32_t inst) {
    if (!b || inst < -1 || inst >= b->n) return FLOU_ERR_ARG;
    b->skip_done_inst = inst;
    drop_graph(b);
    return FLOU_OK;
}

}  // extern "C"
