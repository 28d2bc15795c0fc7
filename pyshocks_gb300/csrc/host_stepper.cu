// Host-resident batches: the state starts and ends in host memory.
//
// The batch is split by instance into chunks of about equal cell counts, each
// with its own plan and device buffers. For chunk c the host-to-device copy
// runs on one copy stream, the reset and steps on one of two compute streams
// (after the copy's event), and the device-to-host copy on a second copy
// stream (after the steps' event), so the copies of one chunk overlap the
// steps of the others and the two copy directions overlap each other. With
// pinned host buffers the call costs about the steps plus one chunk's copies;
// with pageable buffers the CUDA runtime stages the copies and they overlap less.
//
// Every instance is independent (its own dt from its own wave-speed maximum),
// so the result is bit-identical to one plan over the whole batch.

#include "shocks.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <new>
#include <vector>

struct shk_host_stepper {
    int nchunks = 0;
    size_t elem = 8;
    std::vector<shk_plan*> plans;
    std::vector<int64_t> cell0;  // first packed cell of each chunk, nchunks + 1
    std::vector<int32_t> inst0;  // first instance of each chunk, nchunks + 1
    std::vector<void*> ua, ub;   // device state buffers of each chunk
    cudaStream_t h2d = nullptr, d2h = nullptr, comp[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> ev_in, ev_done;
    cudaEvent_t ev_start = nullptr, ev_end[3] = {nullptr, nullptr, nullptr};
};

namespace {

int check(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libshocks: CUDA error %s\n", cudaGetErrorString(e));
        return SHK_ECUDA;
    }
    return SHK_OK;
}

#define HS_CUDA(call)                   \
    do {                                \
        int _st = check(call);          \
        if (_st != SHK_OK) return _st;  \
    } while (0)

#define HS_OK(call)                     \
    do {                                \
        int _st = (call);               \
        if (_st != SHK_OK) return _st;  \
    } while (0)

// instance boundaries of nchunks chunks of about equal cell counts
std::vector<int32_t> split_instances(int32_t batch, const int64_t* off, int nchunks) {
    std::vector<int32_t> cut{0};
    const int64_t total = off[batch] - off[0];
    for (int c = 1; c < nchunks; ++c) {
        const int64_t target = off[0] + total * c / nchunks;
        int32_t b = static_cast<int32_t>(std::lower_bound(off, off + batch + 1, target) - off);
        b = std::max(b, cut.back() + 1);
        if (b >= batch) break;
        cut.push_back(b);
    }
    cut.push_back(batch);
    return cut;
}

}  // namespace

extern "C" {

int shk_host_stepper_destroy(shk_host_stepper* hs) {
    if (!hs) return SHK_OK;
    for (shk_plan* p : hs->plans) shk_plan_destroy(p);
    for (void* p : hs->ua) if (p) cudaFree(p);
    for (void* p : hs->ub) if (p) cudaFree(p);
    for (cudaEvent_t e : hs->ev_in) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : hs->ev_done) if (e) cudaEventDestroy(e);
    if (hs->ev_start) cudaEventDestroy(hs->ev_start);
    for (cudaEvent_t e : hs->ev_end) if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {hs->h2d, hs->d2h, hs->comp[0], hs->comp[1]})
        if (s) cudaStreamDestroy(s);
    delete hs;
    return SHK_OK;
}

int shk_host_stepper_create(const shk_scheme* scheme, int32_t batch, const int64_t* h_offsets,
                            const double* h_dx, const double* h_cfl, double theta,
                            const shk_plan_opts* opts, int32_t nchunks, shk_host_stepper** out) {
    if (!out) return SHK_EINVAL;
    *out = nullptr;
    if (!scheme || batch <= 0 || !h_offsets || !h_dx || !h_cfl || nchunks < 0) return SHK_EINVAL;
    if (opts && opts->max_steps > 0) return SHK_EINVAL;  // no dt history: forward only
    const int dtype = opts ? opts->dtype : SHK_F64;
    if (dtype != SHK_F64 && dtype != SHK_F32) return SHK_EINVAL;
    if (nchunks == 0) {  // chunks of at least 512 Ki cells, at most 32 of them
        const int64_t total = h_offsets[batch] - h_offsets[0];
        nchunks = static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>(32, total >> 19)));
    }
    const std::vector<int32_t> cut = split_instances(batch, h_offsets, std::min(nchunks, batch));
    auto* hs = new (std::nothrow) shk_host_stepper();
    if (!hs) return SHK_ENOMEM;
    hs->nchunks = static_cast<int>(cut.size()) - 1;
    hs->elem = dtype == SHK_F64 ? sizeof(double) : sizeof(float);
    int st = SHK_OK;
    for (int c = 0; c < hs->nchunks && st == SHK_OK; ++c) {
        const int32_t b0 = cut[c], b1 = cut[c + 1];
        std::vector<int64_t> off(b1 - b0 + 1);
        for (int32_t b = b0; b <= b1; ++b) off[b - b0] = h_offsets[b] - h_offsets[b0];
        shk_plan* p = nullptr;
        st = shk_plan_create(scheme, b1 - b0, off.data(), h_dx + b0, h_cfl + b0, theta, opts, &p);
        if (st != SHK_OK) break;
        hs->plans.push_back(p);
        hs->cell0.push_back(h_offsets[b0] - h_offsets[0]);
        hs->inst0.push_back(b0);
        const size_t bytes = hs->elem * size_t(off.back());
        void *a = nullptr, *b = nullptr;
        if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
            if (a) cudaFree(a);
            st = SHK_ENOMEM;
            break;
        }
        hs->ua.push_back(a);
        hs->ub.push_back(b);
    }
    hs->cell0.push_back(h_offsets[batch] - h_offsets[0]);
    hs->inst0.push_back(batch);
    if (st == SHK_OK) {
        bool ok = cudaStreamCreateWithFlags(&hs->h2d, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&hs->d2h, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&hs->comp[0], cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&hs->comp[1], cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&hs->ev_start, cudaEventDisableTiming) == cudaSuccess;
        for (int i = 0; i < 3 && ok; ++i)
            ok = cudaEventCreateWithFlags(&hs->ev_end[i], cudaEventDisableTiming) == cudaSuccess;
        hs->ev_in.assign(hs->nchunks, nullptr);
        hs->ev_done.assign(hs->nchunks, nullptr);
        for (int c = 0; c < hs->nchunks && ok; ++c)
            ok = cudaEventCreateWithFlags(&hs->ev_in[c], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&hs->ev_done[c], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) st = SHK_ECUDA;
    }
    if (st != SHK_OK) {
        shk_host_stepper_destroy(hs);
        return st;
    }
    *out = hs;
    return SHK_OK;
}

int shk_host_stepper_num_chunks(const shk_host_stepper* hs) { return hs ? hs->nchunks : 0; }

int shk_host_stepper_advance(shk_host_stepper* hs, const void* h_in, void* h_out, int32_t nsteps,
                             void* stream) {
    if (!hs || !h_in || !h_out || nsteps < 0) return SHK_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // everything queued on the caller's stream before this call comes first,
    // and the previous call of this stepper (whatever its stream) has ended
    HS_CUDA(cudaEventRecord(hs->ev_start, st));
    for (cudaEvent_t e : hs->ev_end) HS_CUDA(cudaStreamWaitEvent(hs->h2d, e, 0));
    for (cudaStream_t s : {hs->h2d, hs->d2h, hs->comp[0], hs->comp[1]})
        HS_CUDA(cudaStreamWaitEvent(s, hs->ev_start, 0));
    const auto* in = static_cast<const unsigned char*>(h_in);
    auto* out = static_cast<unsigned char*>(h_out);
    for (int c = 0; c < hs->nchunks; ++c) {
        const size_t at = hs->elem * size_t(hs->cell0[c]);
        const size_t bytes = hs->elem * size_t(hs->cell0[c + 1] - hs->cell0[c]);
        HS_CUDA(cudaMemcpyAsync(hs->ua[c], in + at, bytes, cudaMemcpyHostToDevice, hs->h2d));
        HS_CUDA(cudaEventRecord(hs->ev_in[c], hs->h2d));
    }
    for (int c = 0; c < hs->nchunks; ++c) {
        cudaStream_t cs = hs->comp[c & 1];
        HS_CUDA(cudaStreamWaitEvent(cs, hs->ev_in[c], 0));
        HS_OK(shk_plan_reset(hs->plans[c], hs->ua[c], nullptr, nullptr, cs));
        HS_OK(shk_plan_step(hs->plans[c], hs->ua[c], hs->ub[c], nsteps, cs));
        HS_CUDA(cudaEventRecord(hs->ev_done[c], cs));
        const size_t at = hs->elem * size_t(hs->cell0[c]);
        const size_t bytes = hs->elem * size_t(hs->cell0[c + 1] - hs->cell0[c]);
        HS_CUDA(cudaStreamWaitEvent(hs->d2h, hs->ev_done[c], 0));
        HS_CUDA(cudaMemcpyAsync(out + at, nsteps % 2 ? hs->ub[c] : hs->ua[c], bytes,
                                cudaMemcpyDeviceToHost, hs->d2h));
    }
    // the caller's stream waits for the results and for every internal stream
    HS_CUDA(cudaEventRecord(hs->ev_end[0], hs->d2h));
    HS_CUDA(cudaEventRecord(hs->ev_end[1], hs->comp[0]));
    HS_CUDA(cudaEventRecord(hs->ev_end[2], hs->comp[1]));
    for (cudaEvent_t e : hs->ev_end) HS_CUDA(cudaStreamWaitEvent(st, e, 0));
    return SHK_OK;
}

int shk_host_stepper_set_boundary(shk_host_stepper* hs, int32_t left, int32_t right,
                                  const double* dirichlet, const double* neumann, void* stream) {
    if (!hs) return SHK_EINVAL;
    for (int c = 0; c < hs->nchunks; ++c) {
        const size_t b0 = static_cast<size_t>(hs->inst0[c]);
        HS_OK(shk_plan_set_boundary(hs->plans[c], left, right, dirichlet ? dirichlet + 6 * b0 : nullptr,
                                    neumann ? neumann + 2 * b0 : nullptr, stream));
    }
    return SHK_OK;
}

int shk_host_stepper_status(shk_host_stepper* hs, int32_t* h_status, void* stream) {
    if (!hs || !h_status) return SHK_EINVAL;
    int32_t acc = 0;
    for (shk_plan* p : hs->plans) {
        int32_t s = 0;
        HS_OK(shk_plan_status(p, &s, stream));
        acc |= s;
    }
    *h_status = acc;
    return SHK_OK;
}

}  // extern "C"
