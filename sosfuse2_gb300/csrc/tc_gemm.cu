// Tensor-core BF16 GEMM for sm_103a (tcgen05 + TMA + TMEM) and the elementwise kernels of the warm-start MLP.
//
// C[M x N] = A[M x K] * B[N x K]^T, A and B row-major BF16 (K contiguous), FP32 accumulation in tensor memory.
// One CTA (4 warps) computes a 128 x 128 tile: warp 0 lane 0 streams 128 x 64 tiles of A and B into a 4-stage
// shared-memory ring with TMA (128-byte swizzle); warp 1 lane 0 issues tcgen05.mma (M=128, N=128, K=16, four per
// stage) into a 128-column TMEM accumulator and frees each stage with tcgen05.commit; then all four warps read the
// accumulator back (tcgen05.ld, one TMEM lane quarter per warp) and apply the epilogue. Every mbarrier wait is
// bounded by a clock budget: on expiry the kernel records an error code, skips the rest, frees its TMEM and returns,
// and the host reports E_TC_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/sosb.h"
#include "tc_ptx.cuh"

namespace tc {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 4;
constexpr int TILE_BYTES = BM * BK * 2;  // 16 KB per operand tile
constexpr int STAGE_BYTES = 2 * TILE_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t IDESC = tcx::idesc_bf16(BM, BN);

__device__ unsigned g_error;

using tcx::fence_after;
using tcx::fence_before;
using tcx::mbar_expect_tx;
using tcx::mbar_init;
using tcx::mma_commit;
using tcx::smem_u32;
using tcx::sw128_desc;
using tcx::tmem_ld16;

// Bounded wait on a barrier phase; false (with the error recorded) when the budget runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned code) {
    return tcx::mbar_wait(bar, parity, code, &g_error);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    tcx::mma_f16(tmem, a, b, IDESC, accumulate);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

// epilogues: 0 C = acc (FP32); 1 Z = acc + bias -> C = Z (FP32) and H = gelu(Z) (BF16); 2 C = acc + bias (FP32)
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const __grid_constant__ CUtensorMap ta,
                                                        const __grid_constant__ CUtensorMap tb, int M, int N, int K,
                                                        const float* __restrict__ bias, int epilogue,
                                                        float* __restrict__ cf, __nv_bfloat16* __restrict__ cb) {
    extern __shared__ uint8_t sm_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int ktiles = K / BK;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tcx::tmem_alloc(tmem_slot, BN);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    bool ok = true;
    if (warp == 0) {
        if (lane == 0) {
            for (int kt = 0; kt < ktiles && ok; ++kt) {
                const int s = kt % STAGES;
                if (kt >= STAGES) ok = mbar_wait(&empty[s], ((kt / STAGES) - 1) & 1, 1u);
                if (!ok) break;
                uint8_t* st = sm + s * STAGE_BYTES;
                mbar_expect_tx(&full[s], STAGE_BYTES);
                tma_load_2d(st, &ta, &full[s], kt * BK, m0);
                tma_load_2d(st + TILE_BYTES, &tb, &full[s], kt * BK, n0);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            for (int kt = 0; kt < ktiles && ok; ++kt) {
                const int s = kt % STAGES;
                ok = mbar_wait(&full[s], (kt / STAGES) & 1, 2u);
                if (!ok) break;
                fence_after();
                const uint32_t a = smem_u32(sm + s * STAGE_BYTES);
                const uint32_t b = a + TILE_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk)
                    mma_bf16(tmem, sw128_desc(a + kk * 32), sw128_desc(b + kk * 32), (kt > 0 || kk > 0) ? 1u : 0u);
                mma_commit(&empty[s]);
            }
            mma_commit(done);  // arrives once every MMA issued above has completed
        }
        __syncwarp();
    }
    // epilogue: warp w owns accumulator lanes (rows) 32w .. 32w+31
    const bool have = mbar_wait(done, 0, 4u) && !(g_error & 3u);
    fence_after();
    const int row = m0 + warp * 32 + lane;
    if (have) {
        for (int c = 0; c < BN / 16; ++c) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), v);
            const int col = n0 + c * 16;
            if (row < M) {
                if (epilogue != 0) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] += bias[col + i];
                }
                float4* dst = reinterpret_cast<float4*>(cf + (size_t)row * N + col);
#pragma unroll
                for (int i = 0; i < 4; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                if (epilogue == 1) {
                    __nv_bfloat16* h = cb + (size_t)row * N + col;
#pragma unroll
                    for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16_rn(gelu(v[i]));
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tcx::tmem_dealloc(tmem, BN);
}

// ------------------------------------------------------------------------------- elementwise kernels of the MLP
// dZ = dH * gelu'(Z), gelu'(z) = Phi(z) + z phi(z); written as BF16 for the next GEMMs and FP32 for the bias sums
__global__ void gelu_backward_kernel(const float* __restrict__ dh, const float* __restrict__ z, long long n,
                                     __nv_bfloat16* __restrict__ dz_b, float* __restrict__ dz_f) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float zz = z[i];
        const float d = 0.5f * (1.0f + erff(zz * 0.70710678118654752f)) + zz * 0.39894228040143268f * expf(-0.5f * zz * zz);
        const float g = dh[i] * d;
        dz_f[i] = g;
        dz_b[i] = __float2bfloat16_rn(g);
    }
}

// out[c][r] = in[r][c] (BF16 or FP32 -> BF16), rows x cols
__global__ void transpose_bf16_kernel(const void* __restrict__ in, int in_is_f32, int rows, int cols,
                                      __nv_bfloat16* __restrict__ out) {
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        float v = 0.0f;
        if (r < rows && c < cols)
            v = in_is_f32 ? static_cast<const float*>(in)[(size_t)r * cols + c]
                          : __bfloat162float(static_cast<const __nv_bfloat16*>(in)[(size_t)r * cols + c]);
        tile[j][threadIdx.x] = v;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * rows + r] = __float2bfloat16_rn(tile[threadIdx.x][j]);
    }
}

// column sums of a row-major [rows x cols] FP32 matrix (bias gradients)
__global__ void column_sum_kernel(const float* __restrict__ g, int rows, int cols, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f, comp = 0.0f;
    for (int r = 0; r < rows; ++r) {
        const float y = g[(size_t)r * cols + c] - comp;
        const float t = s + y;
        comp = (t - s) - y;
        s = t;
    }
    out[c] = s;
}

// Adam on FP32 master weights, refreshing the BF16 copy (and optionally its transpose)
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2, float decay, __nv_bfloat16* __restrict__ wb) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float wi = w[i] - lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + decay * w[i]);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

// mean squared error gradient: d = 2 (p - y) / count over valid rows; returns partial sums of squares per block
__global__ void mse_kernel(const float* __restrict__ p, const float* __restrict__ y, long long n, float scale,
                           float* __restrict__ d, float* __restrict__ partial) {
    __shared__ float red[256];
    float s = 0.0f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float e = p[i] - y[i];
        d[i] = 2.0f * e * scale;
        s += e * e;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ in, long long n, __nv_bfloat16* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

// ------------------------------------------------------------------------------- host side
static thread_local std::string t_error;
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_lock;

static int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_error = buf;
    return code;
}

static int encoder() {
    std::lock_guard<std::mutex> guard(g_encode_lock);
    if (g_encode) return 0;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return set_error(2, "E_TMA: cuTensorMapEncodeTiled unavailable");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return 0;
}

// TMA map of a row-major [rows x k] BF16 matrix, boxes of 128 rows x 64 columns, 128-byte swizzle
static int make_map(CUtensorMap* map, const void* ptr, int rows, int k) {
    if (reinterpret_cast<uintptr_t>(ptr) % 16) return set_error(3, "E_ALIGN: operand not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)k * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BM};
    cuuint32_t es[2] = {1, 1};
    const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(4, "E_TMA: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return 0;
}

static int grid_1d(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

}  // namespace tc

using namespace tc;

extern "C" {

const char* sosb_tc_last_error(void) { return t_error.c_str(); }

int sosb_gemm_bf16(const void* A, const void* B, int M, int N, int K, const float* bias, int epilogue, float* c_f32,
                   void* c_bf16, void* stream) {
    t_error.clear();
    if (!A || !B || !c_f32 || M <= 0 || N <= 0 || K <= 0) return set_error(1, "E_SHAPE: null operand or empty GEMM");
    if (M % BM || N % BN || K % BK)
        return set_error(1, "E_SHAPE: M %d and N %d must be multiples of 128, K %d of 64", M, N, K);
    if (epilogue < 0 || epilogue > 2 || (epilogue > 0 && !bias) || (epilogue == 1 && !c_bf16))
        return set_error(1, "E_SHAPE: epilogue %d needs its outputs", epilogue);
    if (int r = encoder()) return r;
    CUtensorMap ta, tb;
    if (int r = make_map(&ta, A, M, K)) return r;
    if (int r = make_map(&tb, B, N, K)) return r;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
            cudaSuccess)
            return set_error(5, "E_CUDA: shared memory attribute");
        attr = true;
    }
    dim3 grid(N / BN, M / BM);
    gemm_bf16_kernel<<<grid, 128, SMEM_BYTES, (cudaStream_t)stream>>>(ta, tb, M, N, K, bias, epilogue, c_f32,
                                                                       static_cast<__nv_bfloat16*>(c_bf16));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(6, "E_CUDA: %s", cudaGetErrorString(e));
    return 0;
}

int sosb_tc_check(void* stream) {
    t_error.clear();
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return set_error(6, "E_CUDA: %s", cudaGetErrorString(e));
    unsigned flags = 0;
    e = cudaMemcpyFromSymbol(&flags, g_error, sizeof flags);
    if (e != cudaSuccess) return set_error(6, "E_CUDA: %s", cudaGetErrorString(e));
    if (flags) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_error, &zero, sizeof zero);
        return set_error(7, "E_TC_TIMEOUT: a tensor-core GEMM wait ran out (flags %u)", flags);
    }
    return 0;
}

int sosb_mlp_gelu_backward(const float* dh, const float* z, long long n, void* dz_bf16, float* dz_f32, void* stream) {
    gelu_backward_kernel<<<grid_1d(n), 256, 0, (cudaStream_t)stream>>>(dh, z, n, static_cast<__nv_bfloat16*>(dz_bf16),
                                                                        dz_f32);
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: gelu backward");
}

int sosb_mlp_transpose(const void* in, int in_is_f32, int rows, int cols, void* out_bf16, void* stream) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    transpose_bf16_kernel<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(in, in_is_f32, rows, cols,
                                                                           static_cast<__nv_bfloat16*>(out_bf16));
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: transpose");
}

int sosb_mlp_column_sum(const float* g, int rows, int cols, float* out, void* stream) {
    column_sum_kernel<<<(cols + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g, rows, cols, out);
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: column sum");
}

int sosb_mlp_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                  int step, float decay, void* w_bf16, void* stream) {
    const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
    adam_kernel<<<grid_1d(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2, decay,
                                                               static_cast<__nv_bfloat16*>(w_bf16));
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: adam");
}

int sosb_mlp_mse(const float* p, const float* y, long long n, float scale, float* d, float* partial, int blocks,
                 void* stream) {
    mse_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(p, y, n, scale, d, partial);
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: mse");
}

int sosb_mlp_to_bf16(const float* in, long long n, void* out, void* stream) {
    f32_to_bf16_kernel<<<grid_1d(n), 256, 0, (cudaStream_t)stream>>>(in, n, static_cast<__nv_bfloat16*>(out));
    return cudaGetLastError() == cudaSuccess ? 0 : set_error(6, "E_CUDA: bf16 conversion");
}

}  // extern "C"
