// PCA projection + quantisation (PCACompress, data_tools/ANNs/data_proc/PCACompress.cpp:21-83
// over data_tools/ANNs/data_proc/base/matrix.h:25-125) and the FmtConv conversions
// (data_tools/ANNs/data_proc/FmtConv.cpp:63-131) on the GPU.
//
// values[j] = bias[j] - mips_distance(mat[j], x): the dot product is summed in index order
// in fp32 with separately rounded products, which is the reference's expression as
// written (point.h:148-156); each thread keeps that order for its outputs, so the codes
// are bit-identical to a build of the reference without fast-math reassociation.  The
// work (2 x n x d_in x d_out, 16 GFLOP for 1M x 128 -> 64) is small next to the file
// I/O around it; tensor-core MMA would change the summation order and move codes that
// sit on a quantisation boundary.
//
// Quantisation (matrix.h:99-125): code = int((v + 1) * 0.5 * 255), float add then double
// products, truncated (the reference's out-of-range conversion is undefined; here it
// saturates), clamped to [0, 255], minus 128 for the signed kinds, shifted right by
// 8 - 8/chunk, masked; for 4-bit output the high nibble of byte i is element 2i+1 and the
// low nibble element 2i.
#include <algorithm>
#include <cstring>
#include <string>

#include "internal.h"

namespace nbpg {

constexpr int PCA_PTS = 32;    // points per CTA
constexpr int PCA_OUTS = 64;   // outputs per CTA
constexpr int PCA_THREADS = 256;
constexpr uint32_t PCA_MAX_DIN = 576;  // shared memory: d_in x 384 B + 8 KB

enum PcaIn : int { PIN_F32 = 0, PIN_U8 = 1, PIN_I8 = 2 };

template <int IN>
__device__ __forceinline__ float load_in(const void *x, uint64_t i)
{
    if constexpr (IN == PIN_F32) return static_cast<const float *>(x)[i];
    else if constexpr (IN == PIN_U8) return float(static_cast<const uint8_t *>(x)[i]);
    else return float(static_cast<const int8_t *>(x)[i]);
}

__device__ __forceinline__ int quant_code(float v)
{
    const double t = __dmul_rn(__dmul_rn(double(__fadd_rn(v, 1.0f)), 0.5), 255.0);
    return __double2int_rz(t);  // saturates; NaN gives 0, which clamps like the low end
}

// grid (ceil(n / 32), ceil(d_out / 64)); out_kind: 0 f32, 1 u8, 2 i8, 3 u4, 4 i4
template <int IN>
__global__ void __launch_bounds__(PCA_THREADS) pca_kernel(const void *x, uint64_t n, uint32_t d_in, const float *mat,
                                                         const float *bias, uint32_t d_out, uint32_t out_kind,
                                                         void *out)
{
    extern __shared__ float sm[];
    float *mT = sm;                                   // [d_in][64]
    float *xs = mT + size_t(d_in) * PCA_OUTS;         // [32][d_in]
    float *vals = xs + size_t(PCA_PTS) * d_in;        // [32][64]
    const int tid = threadIdx.x;
    const uint32_t j0 = blockIdx.y * PCA_OUTS;
    const uint64_t p0 = uint64_t(blockIdx.x) * PCA_PTS;
    for (uint32_t e = tid; e < d_in * PCA_OUTS; e += PCA_THREADS) {
        const uint32_t c = e % PCA_OUTS, i = e / PCA_OUTS;
        mT[e] = j0 + c < d_out ? mat[size_t(j0 + c) * d_in + i] : 0.0f;
    }
    for (uint32_t e = tid; e < PCA_PTS * d_in; e += PCA_THREADS) {
        const uint32_t pl = e / d_in, i = e % d_in;
        xs[e] = p0 + pl < n ? load_in<IN>(x, (p0 + pl) * d_in + i) : 0.0f;
    }
    __syncthreads();

    const int g = tid / PCA_OUTS, c = tid % PCA_OUTS;  // 4 groups of 8 points
    float acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0f;
    for (uint32_t i = 0; i < d_in; ++i) {
        const float m = mT[i * PCA_OUTS + c];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = __fadd_rn(acc[q], __fmul_rn(m, xs[(g * 8 + q) * d_in + i]));
    }
    const uint32_t j = j0 + c;
    const float b = j < d_out ? bias[j] : 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float v = __fadd_rn(b, acc[q]);  // bias - (-dot)
        const uint64_t p = p0 + g * 8 + q;
        if (out_kind == 0) {
            if (p < n && j < d_out) static_cast<float *>(out)[p * d_out + j] = v;
        } else {
            vals[(g * 8 + q) * PCA_OUTS + c] = v;
        }
    }
    if (out_kind == 0) return;
    __syncthreads();
    const uint32_t chunk = out_kind >= 3 ? 2 : 1;
    const int delta = (out_kind == 2 || out_kind == 4) ? 128 : 0;
    const int offset = 8 - 8 / int(chunk), mask = (1 << (8 / chunk)) - 1;
    const uint32_t out_dims = d_out / chunk, bpp = PCA_OUTS / chunk;
    for (uint32_t e = tid; e < PCA_PTS * bpp; e += PCA_THREADS) {
        const uint32_t pl = e / bpp, bi = e % bpp;
        const uint32_t ob = j0 / chunk + bi;
        const uint64_t p = p0 + pl;
        if (p >= n || ob >= out_dims) continue;
        uint32_t res = 0;
        for (uint32_t jj = 0; jj < chunk; ++jj) {
            const float v = vals[pl * PCA_OUTS + (bi + 1) * chunk - 1 - jj];
            res = (res << (8 / chunk)) & 0xFFu;
            int ti = quant_code(v);
            ti = (min(max(ti, 0), 255) - delta) >> offset;
            res = (res + uint32_t(ti & mask)) & 0xFFu;
        }
        static_cast<uint8_t *>(out)[p * out_dims + ob] = uint8_t(res);
    }
}

// FmtConv u8bin2u4bin: byte j = (row[2j+1] & 0xF0) + (row[2j] >> 4); odd last element dropped
__global__ void u8_to_u4_kernel(const uint8_t *rows, uint64_t n, uint32_t dims, uint8_t *out)
{
    const uint32_t half = dims >> 1;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < n * half; e += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t p = e / half, j = e % half;
        out[e] = uint8_t((rows[p * dims + 2 * j + 1] & 0xF0) + (rows[p * dims + 2 * j] >> 4));
    }
}

// FmtConv fbin2u8bin: static_cast<unsigned char>(v) for 0 <= v < 256; *bad set otherwise
__global__ void f32_to_u8_kernel(const float *rows, uint64_t count, uint8_t *out, uint32_t *bad)
{
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < count; e += uint64_t(gridDim.x) * blockDim.x) {
        const float v = rows[e];
        if (!(v >= 0.0f && v < 256.0f)) {
            atomicExch(bad, 1u);
            out[e] = 0;
        } else {
            out[e] = uint8_t(__float2uint_rz(v));
        }
    }
}

static size_t pca_smem(uint32_t d_in)
{
    return (size_t(d_in) * PCA_OUTS + size_t(PCA_PTS) * d_in + PCA_PTS * PCA_OUTS) * sizeof(float);
}

static uint32_t out_width(uint32_t out_dtype, uint32_t d_out)
{
    return (out_dtype == NBPG_U4 || out_dtype == NBPG_I4) ? d_out / 2 : d_out;
}

static int out_kind_of(uint32_t out_dtype)
{
    switch (out_dtype) {
    case NBPG_F32: return 0;
    case NBPG_U8: return 1;
    case NBPG_I8: return 2;
    case NBPG_U4: return 3;
    default: return 4;
    }
}

static nbpg_status launch_pca(uint32_t in_dtype, const void *d_x, uint64_t n, uint32_t d_in, const float *d_mat,
                              const float *d_bias, uint32_t d_out, uint32_t out_dtype, void *d_out_rows,
                              cudaStream_t st)
{
    const size_t smem = pca_smem(d_in);
    const dim3 grid(uint32_t((n + PCA_PTS - 1) / PCA_PTS), (d_out + PCA_OUTS - 1) / PCA_OUTS);
    const uint32_t kind = uint32_t(out_kind_of(out_dtype));
    cudaError_t e;
    switch (in_dtype) {
    case NBPG_F32:
        e = cudaFuncSetAttribute(pca_kernel<PIN_F32>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e == cudaSuccess)
            pca_kernel<PIN_F32><<<grid, PCA_THREADS, smem, st>>>(d_x, n, d_in, d_mat, d_bias, d_out, kind, d_out_rows);
        break;
    case NBPG_U8:
        e = cudaFuncSetAttribute(pca_kernel<PIN_U8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e == cudaSuccess)
            pca_kernel<PIN_U8><<<grid, PCA_THREADS, smem, st>>>(d_x, n, d_in, d_mat, d_bias, d_out, kind, d_out_rows);
        break;
    default:
        e = cudaFuncSetAttribute(pca_kernel<PIN_I8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e == cudaSuccess)
            pca_kernel<PIN_I8><<<grid, PCA_THREADS, smem, st>>>(d_x, n, d_in, d_mat, d_bias, d_out, kind, d_out_rows);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_pca_encode: ") + cudaGetErrorString(e));
        return NBPG_ERR_CUDA;
    }
    return NBPG_OK;
}

static nbpg_status check_pca_args(uint32_t in_dtype, uint64_t n, uint32_t d_in, uint32_t d_out, uint32_t out_dtype)
{
    NBPG_CHECK_ARG(in_dtype == NBPG_F32 || in_dtype == NBPG_U8 || in_dtype == NBPG_I8, "input rows must be f32, u8 or i8");
    NBPG_CHECK_ARG(out_dtype <= NBPG_F32, "bad output type");
    NBPG_CHECK_ARG(d_in >= 1 && d_in <= PCA_MAX_DIN, "d_in must be in [1, 576]");
    NBPG_CHECK_ARG(d_out >= 1, "d_out must be >= 1");
    NBPG_CHECK_ARG(!(out_dtype == NBPG_U4 || out_dtype == NBPG_I4) || d_out % 2 == 0,
                   "4-bit output needs an even d_out");
    NBPG_CHECK_ARG(n < (uint64_t(1) << 40), "too many rows");
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_pca_encode_device(uint32_t in_dtype, const void *d_rows, uint64_t n, uint32_t d_in,
                                              const float *d_mat, const float *d_bias, uint32_t d_out,
                                              uint32_t out_dtype, void *d_out_rows, void *stream)
{
    NBPG_CHECK_ARG(d_rows && d_mat && d_bias && d_out_rows, "null argument");
    const nbpg_status s = check_pca_args(in_dtype, n, d_in, d_out, out_dtype);
    if (s != NBPG_OK || n == 0) return s;
    return launch_pca(in_dtype, d_rows, n, d_in, d_mat, d_bias, d_out, out_dtype, d_out_rows,
                      static_cast<cudaStream_t>(stream));
}

// Host buffers; rows stream through the device in blocks of at most 4M rows.
extern "C" nbpg_status nbpg_pca_encode(uint32_t in_dtype, const void *rows, uint64_t n, uint32_t d_in,
                                       const float *mat, const float *bias, uint32_t d_out, uint32_t out_dtype,
                                       void *out, int32_t device)
{
    NBPG_CHECK_ARG(rows && mat && out, "null argument");
    nbpg_status s = check_pca_args(in_dtype, n, d_in, d_out, out_dtype);
    if (s != NBPG_OK || n == 0) return s;
    NBPG_CUDA_TRY(cudaSetDevice(device));
    const size_t in_b = in_dtype == NBPG_F32 ? 4 : 1;
    const size_t out_b = (out_dtype == NBPG_F32 ? 4 : 1) * size_t(out_width(out_dtype, d_out));
    const uint64_t blk = std::min<uint64_t>(n, uint64_t(1) << 22);
    cudaStream_t st;
    NBPG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    void *dx = nullptr, *dy = nullptr;
    float *dm = nullptr, *db = nullptr;
    cudaError_t e = cudaMalloc(&dx, blk * d_in * in_b);
    if (e == cudaSuccess) e = cudaMalloc(&dy, blk * out_b);
    if (e == cudaSuccess) e = cudaMalloc(&dm, size_t(d_out) * d_in * 4);
    if (e == cudaSuccess) e = cudaMalloc(&db, size_t(d_out) * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dm, mat, size_t(d_out) * d_in * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        if (bias) e = cudaMemcpyAsync(db, bias, size_t(d_out) * 4, cudaMemcpyHostToDevice, st);
        else e = cudaMemsetAsync(db, 0, size_t(d_out) * 4, st);
    }
    for (uint64_t p = 0; e == cudaSuccess && s == NBPG_OK && p < n; p += blk) {
        const uint64_t cnt = std::min<uint64_t>(blk, n - p);
        e = cudaMemcpyAsync(dx, static_cast<const uint8_t *>(rows) + p * d_in * in_b, cnt * d_in * in_b,
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) s = launch_pca(in_dtype, dx, cnt, d_in, dm, db, d_out, out_dtype, dy, st);
        if (e == cudaSuccess && s == NBPG_OK)
            e = cudaMemcpyAsync(static_cast<uint8_t *>(out) + p * out_b, dy, cnt * out_b, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess && s == NBPG_OK) {
        set_error(std::string("nbpg_pca_encode: ") + cudaGetErrorString(e));
        s = e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    }
    cudaStreamSynchronize(st);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dm);
    cudaFree(db);
    cudaStreamDestroy(st);
    return s;
}

extern "C" nbpg_status nbpg_u8_to_u4(const uint8_t *rows, uint64_t n, uint32_t dims, uint8_t *out, int32_t device)
{
    NBPG_CHECK_ARG(rows && out, "null argument");
    NBPG_CHECK_ARG(dims >= 2, "dims must be >= 2");
    if (n == 0) return NBPG_OK;
    NBPG_CUDA_TRY(cudaSetDevice(device));
    uint8_t *dx = nullptr, *dy = nullptr;
    const size_t half = dims >> 1;
    nbpg_status s = NBPG_OK;
    cudaError_t e = cudaMalloc(&dx, n * dims);
    if (e == cudaSuccess) e = cudaMalloc(&dy, n * half);
    if (e == cudaSuccess) e = cudaMemcpy(dx, rows, n * dims, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        u8_to_u4_kernel<<<1024, 256>>>(dx, n, dims, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dy, n * half, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_u8_to_u4: ") + cudaGetErrorString(e));
        s = e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    }
    cudaFree(dx);
    cudaFree(dy);
    return s;
}

extern "C" nbpg_status nbpg_f32_to_u8(const float *rows, uint64_t n, uint32_t dims, uint8_t *out, int32_t device)
{
    NBPG_CHECK_ARG(rows && out, "null argument");
    if (n == 0 || dims == 0) return NBPG_OK;
    NBPG_CUDA_TRY(cudaSetDevice(device));
    float *dx = nullptr;
    uint8_t *dy = nullptr;
    uint32_t *dbad = nullptr, bad = 0;
    nbpg_status s = NBPG_OK;
    const uint64_t cnt = n * dims;
    cudaError_t e = cudaMalloc(&dx, cnt * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dy, cnt);
    if (e == cudaSuccess) e = cudaMalloc(&dbad, 4);
    if (e == cudaSuccess) e = cudaMemset(dbad, 0, 4);
    if (e == cudaSuccess) e = cudaMemcpy(dx, rows, cnt * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        f32_to_u8_kernel<<<1024, 256>>>(dx, cnt, dy, dbad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dy, cnt, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&bad, dbad, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_f32_to_u8: ") + cudaGetErrorString(e));
        s = e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    } else if (bad) {
        set_error("nbpg_f32_to_u8: a value lies outside [0, 256)");
        s = NBPG_ERR_INVALID_ARG;
    }
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dbad);
    return s;
}
