// pipeline.cu -- batched calls on HOST buffers, streamed through the device in
// chunks.
//
// The reference moves a batch to the device with one synchronous copy
// (DTensor's host-vector constructor, include/tensor.cuh:875-884, through
// upload, include/tensor.cuh:1129-1145), runs the cuBLAS / cuSOLVER call, and
// copies the result back (download, include/tensor.cuh:1147-1154).  On a GB300 the host
// link (NVLink-C2C to the Grace CPU) carries ~210 GB/s host-to-device and
// ~190 GB/s device-to-host at the same time, while the batched kernels run at
// several TB/s, so the copies dominate such a step.  Here the batch is split
// into chunks that rotate over a few worker streams: chunk c's inputs are
// copied in while chunk c-1 computes and chunk c-2's results are copied out,
// so both copy directions and the kernels overlap and the step approaches
// the time of the larger copy.  Device staging buffers belong to the
// pipeline object (a few chunks, not the whole batch) and only grow.
//
// Host buffers should be page-locked (cudaHostAlloc / cudaHostRegister) for
// the copies to be asynchronous; pageable memory gives the same results with
// copies the runtime stages synchronously.
#include <vector>

#include "common.cuh"

struct gbla_stream_pipeline {
    struct Worker {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        void *buf = nullptr;
        size_t bytes = 0;
    };
    std::vector<Worker> workers;
    cudaEvent_t start = nullptr;
    int device = -1;
};

namespace gbla {

namespace {

// Copy `count` matrices of `elems` floats between a strided and a packed layout.
gbla_status copy_matrices(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int64_t count,
                          cudaMemcpyKind kind, cudaStream_t st) {
    if (count <= 0 || width == 0) return GBLA_SUCCESS;
    cudaError_t e;
    if (dpitch == width && spitch == width)
        e = cudaMemcpyAsync(dst, src, width * (size_t)count, kind, st);
    else
        e = cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, (size_t)count, kind, st);
    return from_cuda(e);
}

// Make every worker's staging buffer at least `bytes` long.
gbla_status reserve(gbla_stream_pipeline *p, size_t bytes) {
    for (auto &w : p->workers) {
        if (w.bytes >= bytes) continue;
        if (w.buf) {
            cudaError_t e = cudaStreamSynchronize(w.stream);  // earlier chunks may still use it
            if (e != cudaSuccess) return from_cuda(e);
            cudaFree(w.buf);
            w.buf = nullptr;
            w.bytes = 0;
        }
        cudaError_t e = cudaMalloc(&w.buf, bytes);
        if (e != cudaSuccess) {
            w.buf = nullptr;
            return from_cuda(e);
        }
        w.bytes = bytes;
    }
    return GBLA_SUCCESS;
}

// Fork the workers from the caller's stream.
gbla_status fork(gbla_stream_pipeline *p, cudaStream_t st) {
    cudaError_t e = cudaEventRecord(p->start, st);
    for (auto &w : p->workers)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(w.stream, p->start, 0);
    return from_cuda(e);
}

// Join the workers back into the caller's stream.
gbla_status join(gbla_stream_pipeline *p, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    for (auto &w : p->workers) {
        if (e == cudaSuccess) e = cudaEventRecord(w.done, w.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, w.done, 0);
    }
    return from_cuda(e);
}

int64_t default_chunk(int64_t batch, int64_t min_chunk) {
    int64_t c = (batch + 7) / 8;  // eight chunks: fill and drain cost about one chunk's compute + copy-out
    if (c < min_chunk) c = min_chunk;
    return c < batch ? c : batch;
}

char *align256(void *p) { return reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255)); }

// The pipeline's streams and buffers belong to the device it was created on.
bool on_own_device(const gbla_stream_pipeline *p) {
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess && dev == p->device;
}

}  // namespace

}  // namespace gbla

using namespace gbla;

GBLA_API gbla_status gbla_pipeline_create(int streams, gbla_stream_pipeline **out) {
    if (!out || streams < 1 || streams > 8) return GBLA_INVALID_VALUE;
    *out = nullptr;
    auto *p = new gbla_stream_pipeline();
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->start, cudaEventDisableTiming);
    p->workers.resize(streams);
    for (auto &w : p->workers) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        gbla_pipeline_destroy(p);
        return from_cuda(e);
    }
    *out = p;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_pipeline_destroy(gbla_stream_pipeline *p) {
    if (!p) return GBLA_SUCCESS;
    for (auto &w : p->workers) {
        if (w.stream) cudaStreamSynchronize(w.stream);
        if (w.buf) cudaFree(w.buf);
        if (w.done) cudaEventDestroy(w.done);
        if (w.stream) cudaStreamDestroy(w.stream);
    }
    if (p->start) cudaEventDestroy(p->start);
    delete p;
    return GBLA_SUCCESS;
}

GBLA_API gbla_status gbla_sgemm_batched_host(gbla_stream_pipeline *p, int m, int n, int k, float alpha,
                                             const float *A, int64_t sA, const float *B, int64_t sB, float beta,
                                             float *Cm, int64_t sC, int batch, gbla_gemm_mode mode, int chunk,
                                             cudaStream_t st) {
    if (!p || m < 0 || n < 0 || k < 0 || batch < 0 || chunk < 0) return GBLA_INVALID_VALUE;
    if (batch == 0 || m == 0 || n == 0) return GBLA_SUCCESS;
    if (!on_own_device(p)) return GBLA_INVALID_VALUE;
    const int64_t ea = (int64_t)m * k, eb = (int64_t)k * n, ec = (int64_t)m * n;
    if ((ea > 0 && (!A || sA < ea)) || (eb > 0 && (!B || sB < eb)) || !Cm || sC < ec) return GBLA_INVALID_VALUE;
    const int64_t cs = chunk > 0 ? (chunk < batch ? chunk : batch) : default_chunk(batch, 1024);
    const size_t ba = round_up(cs * ea * 4, 256), bb = round_up(cs * eb * 4, 256), bc = round_up(cs * ec * 4, 256);
    gbla_status s = reserve(p, ba + bb + bc + 256);
    if (s == GBLA_SUCCESS) s = fork(p, st);
    const size_t W = p->workers.size();
    for (int64_t c0 = 0, i = 0; s == GBLA_SUCCESS && c0 < batch; c0 += cs, i++) {
        const int64_t cnt = (batch - c0) < cs ? (batch - c0) : cs;
        auto &w = p->workers[i % W];
        char *base = align256(w.buf);
        float *dA = reinterpret_cast<float *>(base), *dB = reinterpret_cast<float *>(base + ba),
              *dC = reinterpret_cast<float *>(base + ba + bb);
        s = copy_matrices(dA, ea * 4, A + c0 * sA, sA * 4, ea * 4, cnt, cudaMemcpyHostToDevice, w.stream);
        if (s == GBLA_SUCCESS)
            s = copy_matrices(dB, eb * 4, B + c0 * sB, sB * 4, eb * 4, cnt, cudaMemcpyHostToDevice, w.stream);
        if (s == GBLA_SUCCESS && beta != 0.f)
            s = copy_matrices(dC, ec * 4, Cm + c0 * sC, sC * 4, ec * 4, cnt, cudaMemcpyHostToDevice, w.stream);
        if (s == GBLA_SUCCESS)
            s = gbla_sgemm_batched(m, n, k, alpha, dA, ea, dB, eb, beta, dC, ec, (int)cnt, mode, w.stream);
        if (s == GBLA_SUCCESS)
            s = copy_matrices(Cm + c0 * sC, sC * 4, dC, ec * 4, ec * 4, cnt, cudaMemcpyDeviceToHost, w.stream);
    }
    gbla_status sj = join(p, st);
    return s != GBLA_SUCCESS ? s : sj;
}

GBLA_API gbla_status gbla_sgels_batched_host(gbla_stream_pipeline *p, int m, int n, int nrhs, const float *A,
                                             int64_t sA, float *F, const float *B, int64_t sB, float *X, int *info,
                                             int refine, int batch, int chunk, cudaStream_t st) {
    if (!p || m < 0 || n < 0 || nrhs < 0 || batch < 0 || chunk < 0 || refine < 0 || m < n) return GBLA_INVALID_VALUE;
    if (batch == 0 || n == 0) return GBLA_SUCCESS;
    if (!on_own_device(p)) return GBLA_INVALID_VALUE;
    const int64_t ea = (int64_t)m * n, eb = (int64_t)m * nrhs;
    if (!A || sA < ea || (nrhs > 0 && (!B || !X || sB < eb))) return GBLA_INVALID_VALUE;
    if (m > 128 || n > 32) return GBLA_NOT_SUPPORTED;
    const int64_t cs = chunk > 0 ? (chunk < batch ? chunk : batch) : default_chunk(batch, 1024);
    const size_t ba = round_up(cs * ea * 4, 256), bb = round_up(cs * eb * 4, 256), bi = round_up(cs * 4, 256);
    gbla_status s = reserve(p, ba + bb + bi + 256);
    if (s == GBLA_SUCCESS) s = fork(p, st);
    const size_t W = p->workers.size();
    for (int64_t c0 = 0, i = 0; s == GBLA_SUCCESS && c0 < batch; c0 += cs, i++) {
        const int64_t cnt = (batch - c0) < cs ? (batch - c0) : cs;
        auto &w = p->workers[i % W];
        char *base = align256(w.buf);
        float *dA = reinterpret_cast<float *>(base), *dB = reinterpret_cast<float *>(base + ba);
        int *dI = reinterpret_cast<int *>(base + ba + bb);
        s = copy_matrices(dA, ea * 4, A + c0 * sA, sA * 4, ea * 4, cnt, cudaMemcpyHostToDevice, w.stream);
        if (s == GBLA_SUCCESS && nrhs > 0)
            s = copy_matrices(dB, eb * 4, B + c0 * sB, sB * 4, eb * 4, cnt, cudaMemcpyHostToDevice, w.stream);
        if (s == GBLA_SUCCESS)
            s = gbla_sgels_batched(m, n, nrhs, dA, ea, dB, eb, dI, refine, (int)cnt, w.stream);
        if (s == GBLA_SUCCESS && nrhs > 0)
            s = copy_matrices(X + c0 * sB, sB * 4, dB, eb * 4, eb * 4, cnt, cudaMemcpyDeviceToHost, w.stream);
        if (s == GBLA_SUCCESS && F)
            s = copy_matrices(F + c0 * sA, sA * 4, dA, ea * 4, ea * 4, cnt, cudaMemcpyDeviceToHost, w.stream);
        if (s == GBLA_SUCCESS && info)
            s = from_cuda(cudaMemcpyAsync(info + c0, dI, cnt * sizeof(int), cudaMemcpyDeviceToHost, w.stream));
    }
    gbla_status sj = join(p, st);
    return s != GBLA_SUCCESS ? s : sj;
}
