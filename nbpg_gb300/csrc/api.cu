// C ABI: index handles, data upload/download, error reporting.
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace nbpg {
static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace nbpg

using namespace nbpg;

extern "C" const char *nbpg_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *nbpg_version(void) { return "nbpg_gb300 0.1 (sm_103a)"; }

static uint32_t elem_bytes_row(uint32_t dtype, uint32_t dims)
{
    return dtype == NBPG_F32 ? dims * 4 : dims;  // packed 4-bit: dims already counts bytes
}

extern "C" nbpg_status nbpg_index_create(const nbpg_index_desc *desc, nbpg_index **out)
{
    NBPG_CHECK_ARG(desc && out, "null argument");
    NBPG_CHECK_ARG(desc->dtype <= NBPG_I4, "graph indexes take u8/i8/u4/i4 vectors");
    NBPG_CHECK_ARG(desc->metric <= NBPG_IP, "unknown metric");
    NBPG_CHECK_ARG(desc->dims >= 1 && desc->n >= 1 && desc->n < 0xFFFFFFFFull, "bad sizes");
    NBPG_CHECK_ARG(desc->max_degree >= 1 && desc->max_degree <= 128, "max_degree must be in [1, 128]");
    *out = nullptr;
    NBPG_CUDA_TRY(cudaSetDevice(desc->device));
    auto *idx = new nbpg_index();
    idx->desc = *desc;
    idx->row_bytes = elem_bytes_row(desc->dtype, desc->dims);
    idx->row_stride = round_up(idx->row_bytes, 16);
    idx->gstride = round_up(desc->max_degree + 1, 4);
    cudaDeviceProp prop{};
    cudaError_t e = cudaGetDeviceProperties(&prop, desc->device);
    if (e != cudaSuccess) { delete idx; set_error(cudaGetErrorString(e)); return NBPG_ERR_CUDA; }
    idx->sm_count = prop.multiProcessorCount;
    idx->smem_optin = prop.sharedMemPerBlockOptin;
    e = cudaStreamCreateWithFlags(&idx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&idx->d_points, size_t(desc->n) * idx->row_stride);
    if (e == cudaSuccess) e = cudaMalloc(&idx->d_graph, size_t(desc->n) * idx->gstride * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(idx->d_points, 0, size_t(desc->n) * idx->row_stride, idx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(idx->d_graph, 0, size_t(desc->n) * idx->gstride * 4, idx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(idx->stream);
    if (e != cudaSuccess) {
        set_error(std::string("index allocation: ") + cudaGetErrorString(e));
        nbpg_index_destroy(idx);
        return e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    }
    *out = idx;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_index_destroy(nbpg_index *idx)
{
    if (!idx) return NBPG_OK;
    cudaSetDevice(idx->desc.device);
    if (idx->stream) cudaStreamSynchronize(idx->stream);
    if (idx->d_points) cudaFree(idx->d_points);
    if (idx->d_graph) cudaFree(idx->d_graph);
    if (idx->d_raw) cudaFree(idx->d_raw);
    idx->scratch.release();
    host_call_release(idx->host_call);
    idx->host_call = nullptr;
    for (nbpg::HostCall *c : idx->async_calls) host_call_release(c);
    idx->async_calls.clear();
    for (auto &e : idx->stream_scratch) e.second->release();
    idx->stream_scratch.clear();
    for (DevBuf *b : {&idx->qbuf, &idx->obuf, &idx->ghash, &idx->order_buf}) b->release();
    if (idx->stream) cudaStreamDestroy(idx->stream);
    delete idx;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_index_set_points(nbpg_index *idx, const void *rows, uint64_t first, uint64_t count)
{
    NBPG_CHECK_ARG(idx && (rows || count == 0), "null argument");
    NBPG_CHECK_ARG(first <= idx->desc.n && count <= idx->desc.n - first, "rows out of range");
    if (count == 0) return NBPG_OK;
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(idx->d_points + first * idx->row_stride, idx->row_stride, rows, idx->row_bytes,
                                    idx->row_bytes, count, cudaMemcpyHostToDevice, idx->stream));
    NBPG_CUDA_TRY(cudaStreamSynchronize(idx->stream));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_index_set_graph(nbpg_index *idx, const uint32_t *rows, uint64_t first, uint64_t count)
{
    NBPG_CHECK_ARG(idx && (rows || count == 0), "null argument");
    NBPG_CHECK_ARG(first <= idx->desc.n && count <= idx->desc.n - first, "rows out of range");
    if (count == 0) return NBPG_OK;
    const uint32_t R = idx->desc.max_degree;
    const uint64_t n = idx->desc.n;
    for (uint64_t i = 0; i < count; ++i) {
        const uint32_t *r = rows + i * (R + 1);
        if (r[0] > R) { set_error("graph row degree above max_degree"); return NBPG_ERR_FORMAT; }
        for (uint32_t j = 0; j < r[0]; ++j)
            if (r[1 + j] >= n) { set_error("graph neighbour id out of range"); return NBPG_ERR_FORMAT; }
    }
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    // slots past the degree are zeroed so the device never sees stale ids
    std::vector<uint32_t> tmp(size_t(count) * idx->gstride, 0u);
    for (uint64_t i = 0; i < count; ++i) {
        const uint32_t *r = rows + i * (R + 1);
        std::memcpy(&tmp[i * idx->gstride], r, (1 + r[0]) * sizeof(uint32_t));
    }
    NBPG_CUDA_TRY(cudaMemcpyAsync(idx->d_graph + first * idx->gstride, tmp.data(), tmp.size() * 4,
                                  cudaMemcpyHostToDevice, idx->stream));
    NBPG_CUDA_TRY(cudaStreamSynchronize(idx->stream));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_index_get_graph(const nbpg_index *cidx, uint32_t *rows, uint64_t first, uint64_t count)
{
    auto *idx = const_cast<nbpg_index *>(cidx);
    NBPG_CHECK_ARG(idx && (rows || count == 0), "null argument");
    NBPG_CHECK_ARG(first <= idx->desc.n && count <= idx->desc.n - first, "rows out of range");
    if (count == 0) return NBPG_OK;
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    const uint32_t R = idx->desc.max_degree;
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(rows, (R + 1) * 4, idx->d_graph + first * idx->gstride, idx->gstride * 4,
                                    (R + 1) * 4, count, cudaMemcpyDeviceToHost, idx->stream));
    NBPG_CUDA_TRY(cudaStreamSynchronize(idx->stream));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_index_device_info(const nbpg_index *idx, void **d_points, uint32_t *row_stride,
                                              uint32_t **d_graph, uint32_t *graph_stride)
{
    NBPG_CHECK_ARG(idx, "null index");
    if (d_points) *d_points = idx->d_points;
    if (row_stride) *row_stride = idx->row_stride;
    if (d_graph) *d_graph = idx->d_graph;
    if (graph_stride) *graph_stride = idx->gstride;
    return NBPG_OK;
}
