// fcs_mlp.cu -- the surrogate MLP ensemble (include/fcs_mlp.h): a BF16
// tensor-core GEMM for sm_103a (TMA -> shared memory -> tcgen05.mma ->
// TMEM -> fused epilogue) and the forward, backward and Adam passes built on
// it.  No counterpart in the reference.
//
// One GEMM kernel serves every product of training and inference:
//   D[M][N] = A[M][K] . B[N][K]^T      (A, B BF16 K-major, D FP32 in TMEM)
// with the epilogue selecting what happens to D:
//   EPI_HIDDEN  z = D + b;  h = GELU(z)  -> h (row-major), z, h^T  (BF16)
//   EPI_OUT     y = D + b (optionally de-normalised)   -> FP32 rows
//   EPI_DGRAD   dz = D * GELU'(z)        -> dz (row-major), dz^T  (BF16)
//   EPI_WGRAD   dW += D                  (FP32 atomics; split-K over the batch)
// Layers: forward  h_l = GELU(h_{l-1} W_l^T + b_l)      A = h_{l-1}, B = W_l
//         dgrad    dh_{l-1} = dz_l W_l                 A = dz_l,    B = W_l^T (kept as a copy)
//         wgrad    dW_l = dz_l^T h_{l-1}               A = dz_l^T,  B = h_{l-1}^T
// so every operand is K-major and the transposed activations are written by
// the producing epilogue (their stores are coalesced across the warp).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/fcs_mlp.h"
#include "fcs_mlp_internal.h"
#include "fcs_tc.cuh"

using bf16 = __nv_bfloat16;

namespace fcs {
namespace mlp {

constexpr int BM = 128, BK = 64;
constexpr int kThreads = 192;  // warp 0 TMA, warp 1 TMEM + MMA, warps 2-5 epilogue

enum Epi : int { EPI_HIDDEN = 0, EPI_OUT = 1, EPI_DGRAD = 2, EPI_WGRAD = 3 };

struct GemmArgs {
    int M, N, K;        // rows of A (and D); rows of B (= columns of D); reduction length
    int kSplit;         // K elements per blockIdx.z
    int mode;
    int nValid;         // columns of D that are stored
    const float* bias;  // [N] (HIDDEN, OUT)
    const float* outScale;  // OUT: y = (D + b) * scale + shift (null: no de-normalisation)
    const float* outShift;
    bf16* h; int ldh;   // HIDDEN: GELU output; DGRAD: dz (row-major)
    bf16* z; int ldz;   // HIDDEN: pre-activation out (may be null); DGRAD: pre-activation in
    bf16* t; int ldt;   // HIDDEN: GELU output transposed; DGRAD: dz transposed (may be null)
    float* f; int ldf;  // OUT: FP32 rows; WGRAD: FP32 accumulation target
    int* err;
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ void store16_bf16(bf16* dst, const float (&v)[16]) {
    __align__(16) bf16 tmp[16];
#pragma unroll
    for (int i = 0; i < 16; i++) tmp[i] = __float2bfloat16_rn(v[i]);
    const uint4* s = reinterpret_cast<const uint4*>(tmp);
    uint4* d = reinterpret_cast<uint4*>(dst);
    d[0] = s[0];
    d[1] = s[1];
}

__device__ __forceinline__ void load16_bf16(const bf16* src, float (&v)[16]) {
    __align__(16) bf16 tmp[16];
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(tmp);
    d[0] = s[0];
    d[1] = s[1];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __bfloat162float(tmp[i]);
}

template<int BN, int STAGES>
struct GemmSmem {
    static constexpr int A_BYTES = BM * BK * 2;
    static constexpr int B_BYTES = BN * BK * 2;
    static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr int BYTES = STAGES * STAGE_BYTES + 1024 /* alignment */ + 256 /* barriers */;
};

template<int BN, int STAGES>
__global__ void __launch_bounds__(kThreads, 1)
gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, const GemmArgs a) {
    using S = GemmSmem<BN, STAGES>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * S::STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint32_t* tmemBase = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abortFlag = reinterpret_cast<volatile int*>(tmemBase + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kBeg = blockIdx.z * a.kSplit;
    const int kEnd = min(a.K, kBeg + a.kSplit);
    const int nk = kEnd > kBeg ? (kEnd - kBeg + BK - 1) / BK : 0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(done, 1);
        *abortFlag = 0;
        tc::fence_mbar_init();
        tc::tma_prefetch_map(&mapA);
        tc::tma_prefetch_map(&mapB);
    }
    if (warp == 1) tc::tmem_alloc(tmemBase, BN);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmemBase;

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int i = 0; i < nk; i++) {
            const int s = i % STAGES;
            if (i >= STAGES && !tc::mbar_wait(&empty[s], ((i / STAGES) - 1) & 1, a.err, 1, abortFlag)) break;
            uint8_t* sa = base + s * S::STAGE_BYTES;
            uint8_t* sb = sa + S::A_BYTES;
            tc::mbar_arrive_expect_tx(&full[s], S::STAGE_BYTES);
            tc::tma_load_2d(sa, &mapA, &full[s], kBeg + i * BK, m0);
            tc::tma_load_2d(sb, &mapB, &full[s], kBeg + i * BK, n0);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: 4 x (128 x BN x 16) per 64-wide K chunk
        constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
        for (int i = 0; i < nk; i++) {
            const int s = i % STAGES;
            if (!tc::mbar_wait(&full[s], (i / STAGES) & 1, a.err, 2, abortFlag)) break;
            tc::tc_fence_after();
            const uint32_t sa = tc::smem_u32(base + s * S::STAGE_BYTES);
            const uint32_t sb = sa + S::A_BYTES;
#pragma unroll
            for (int j = 0; j < BK / 16; j++)
                tc::mma_bf16(tmem, tc::desc_k_sw128(sa + 32 * j), tc::desc_k_sw128(sb + 32 * j), idesc,
                             (i | j) != 0);
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(done);
    } else if (warp >= 2) {
        // epilogue: warp (w % 4) owns TMEM lanes 32*(w % 4) .. +31 = rows of the tile
        const int q = warp & 3;
        const bool ok = tc::mbar_wait(done, 0, a.err, 3, abortFlag);
        __syncwarp();
        tc::tc_fence_after();
        const int m = m0 + 32 * q + lane;
        const bool rowOk = ok && m < a.M;
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            __syncwarp();
            tc::tmem_ld16(tmem + (static_cast<uint32_t>(32 * q) << 16) + c0, v);
            if (!rowOk) continue;
            const int nb = n0 + c0;
            if (a.mode == EPI_HIDDEN) {
                float h[16];
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    v[i] += a.bias[nb + i];
                    h[i] = gelu(v[i]);
                }
                store16_bf16(a.h + (size_t)m * a.ldh + nb, h);
                if (a.z) store16_bf16(a.z + (size_t)m * a.ldz + nb, v);
                if (a.t) {
#pragma unroll
                    for (int i = 0; i < 16; i++) a.t[(size_t)(nb + i) * a.ldt + m] = __float2bfloat16_rn(h[i]);
                }
            } else if (a.mode == EPI_OUT) {
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int n = nb + i;
                    if (n < a.nValid) {
                        float y = v[i] + a.bias[n];
                        if (a.outScale) y = fmaf(y, a.outScale[n], a.outShift[n]);
                        a.f[(size_t)m * a.ldf + n] = y;
                    }
                }
            } else if (a.mode == EPI_DGRAD) {
                float z[16];
                load16_bf16(a.z + (size_t)m * a.ldz + nb, z);
#pragma unroll
                for (int i = 0; i < 16; i++) v[i] *= gelu_grad(z[i]);
                store16_bf16(a.h + (size_t)m * a.ldh + nb, v);
                if (a.t) {
#pragma unroll
                    for (int i = 0; i < 16; i++) a.t[(size_t)(nb + i) * a.ldt + m] = __float2bfloat16_rn(v[i]);
                }
            } else {  // EPI_WGRAD
#pragma unroll
                for (int i = 0; i < 16; i++)
                    if (nb + i < a.nValid) atomicAdd(a.f + (size_t)m * a.ldf + nb + i, v[i]);
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, BN);
    }
}

// ---- elementwise kernels ----------------------------------------------------

// X[m][k] = bf16((x[src(m)][k] - mean[k]) * rstd[k]) for k < nIn, 0 for the
// padding up to kPad; optionally the transpose XT[k][m].  src(m) = perm[m]
// (training batches) or m.
__global__ void pack_input_kernel(int n, int nIn, int kPad, const float* x, const long long* perm, long long permOff,
                                  const float* mean, const float* rstd, bf16* X, bf16* XT, int ldT) {
    const long long total = (long long)n * kPad;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(i / kPad), k = (int)(i % kPad);
        float v = 0.f;
        if (k < nIn) {
            const long long src = perm ? perm[permOff + m] : m;
            v = (x[src * nIn + k] - mean[k]) * rstd[k];
        }
        const bf16 b = __float2bfloat16_rn(v);
        X[(size_t)m * kPad + k] = b;
        if (XT) XT[(size_t)k * ldT + m] = b;
    }
}

// d = out - (target - mean) / std over the nOut valid columns; loss += sum d^2;
// dOut = 2 d / (n * nOut) as BF16 rows and transpose (padding columns 0).
__global__ void loss_grad_kernel(int n, int nOut, int nPad, const float* out, const float* target, const long long* perm,
                                 long long permOff, const float* mean, const float* std_, bf16* dOut, bf16* dOutT,
                                 int ldT, float* loss) {
    __shared__ float red[32];
    const long long total = (long long)n * nPad;
    const float scale = 2.f / ((float)n * (float)nOut);
    float acc = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(i / nPad), c = (int)(i % nPad);
        float g = 0.f;
        if (c < nOut) {
            const long long src = perm ? perm[permOff + m] : m;
            const float tn = (target[src * nOut + c] - mean[c]) / std_[c];
            const float d = out[(size_t)m * nPad + c] - tn;
            acc += d * d;
            g = scale * d;
        }
        const bf16 b = __float2bfloat16_rn(g);
        dOut[(size_t)m * nPad + c] = b;
        dOutT[(size_t)c * ldT + m] = b;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(loss, s);
    }
}

// db[r] = sum_m T[r][m]  (one block per row)
__global__ void rowsum_kernel(int rows, int n, const bf16* T, int ldT, float* db) {
    __shared__ float red[32];
    const int r = blockIdx.x;
    if (r >= rows) return;
    float s = 0.f;
    for (int m = threadIdx.x; m < n; m += blockDim.x) s += __bfloat162float(T[(size_t)r * ldT + m]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) db[r] = t;
    }
}

// Adam on one layer (lr > 0) or a plain publish (lr == 0), then the BF16
// copies W[n][k] (ld kPad) and WT[k][n] (ld nPad) of the updated weights.
__global__ void adam_publish_kernel(int nOut, int nIn, int kPad, int nPad, float* W, float* b, float* mW, float* vW,
                                    float* mb, float* vb, const float* gW, const float* gb, float lr, float beta1,
                                    float beta2, float eps, float c1, float c2, bf16* Wbf, bf16* WTbf) {
    const int total = nOut * nIn + nOut;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const bool isW = i < nOut * nIn;
        const int n = isW ? i / nIn : i - nOut * nIn;
        const int k = isW ? i % nIn : 0;
        float* p = isW ? &W[i] : &b[n];
        if (lr > 0.f) {
            const float g = isW ? gW[(size_t)n * kPad + k] : gb[n];
            float* m = isW ? &mW[i] : &mb[n];
            float* v = isW ? &vW[i] : &vb[n];
            const float mi = beta1 * *m + (1.f - beta1) * g;
            const float vi = beta2 * *v + (1.f - beta2) * g * g;
            *m = mi;
            *v = vi;
            *p -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        }
        if (isW) {
            const bf16 w = __float2bfloat16_rn(*p);
            Wbf[(size_t)n * kPad + k] = w;
            WTbf[(size_t)k * nPad + n] = w;
        }
    }
}

// ---- host side -----------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool encoder_ready() {
    if (g_encode) return true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return false;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return true;
}

// BF16 matrix [rows][cols] (row pitch ld elements), box of 64 columns x boxRows
// rows, 128-byte swizzle, zero fill outside the matrix.
bool make_map(CUtensorMap* m, const void* ptr, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t boxRows) {
    if (!encoder_ready()) return false;
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (ld * 2) % 16 || cols % 64) return false;
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {ld * 2};
    cuuint32_t box[2] = {64, boxRows};
    cuuint32_t es[2] = {1, 1};
    return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template<int BN, int STAGES>
cudaError_t launch_gemm_bn(const CUtensorMap& ma, const CUtensorMap& mb, const GemmArgs& a, dim3 grid, cudaStream_t st) {
    static bool attrSet = false;
    const int smem = GemmSmem<BN, STAGES>::BYTES;
    if (!attrSet) {
        cudaError_t e = cudaFuncSetAttribute(gemm_kernel<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attrSet = true;
    }
    gemm_kernel<BN, STAGES><<<grid, kThreads, smem, st>>>(ma, mb, a);
    return cudaGetLastError();
}

// D[M][N] = A[M][K] B[N][K]^T with A (ld lda) and B (ld ldb) BF16 K-major;
// N a multiple of 128, K a multiple of 64; `splits` K slices (WGRAD only).
cudaError_t gemm(const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K, int splits, GemmArgs a,
                 cudaStream_t st) {
    if (M <= 0 || N % 128 || K % 64 || K <= 0) return cudaErrorInvalidValue;
    const int BN = (N % 256 == 0) ? 256 : 128;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda, BM) || !make_map(&mb, B, N, K, ldb, BN)) return cudaErrorInvalidValue;
    splits = std::max(1, std::min(splits, K / BK));
    a.M = M;
    a.N = N;
    a.K = K;
    a.kSplit = ((K / BK + splits - 1) / splits) * BK;
    const int zs = (K + a.kSplit - 1) / a.kSplit;
    dim3 grid((M + BM - 1) / BM, N / BN, zs);
    if (BN == 256) return launch_gemm_bn<256, 2>(ma, mb, a, grid, st);
    return launch_gemm_bn<128, 3>(ma, mb, a, grid, st);
}

int blocks_for(long long n, int block) {
    long long b = (n + block - 1) / block;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}

}  // namespace mlp
}  // namespace fcs

using namespace fcs::mlp;

// ---- the ensemble object ----------------------------------------------------

namespace {

template<class T>
struct DArr {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t want) {
        if (want <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
        if (e == cudaSuccess) {
            n = want;
            e = cudaMemset(p, 0, want * sizeof(T));
            if (e == cudaSuccess) e = cudaDeviceSynchronize();  // before use on non-blocking streams
        }
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct Layer {
    int in, out, kPad, nPad;
    size_t wOff, bOff;     // in the flat parameter vector
    size_t gOff, gbOff;    // in the padded gradient buffers
};

struct Member {
    DArr<float> params, m, v;
    std::vector<DArr<bf16>> W, WT;
    long long step = 0;
};

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

struct fcs_mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    fcs_mlp_shape sh{};
    std::vector<Layer> L;
    int64_t P = 0;
    std::vector<Member> mem;
    DArr<float> inMean, inRstd, outMean, outStd;
    std::vector<float> hInMean, hInStd, hOutMean, hOutStd;
    DArr<float> gW, gb;
    // activations
    DArr<bf16> X, XT, dOut, dOutT, dZT;
    std::vector<DArr<bf16>> Z, H, HT;
    DArr<bf16> dZ[2];
    DArr<float> Out, xDev, yDev, tDev;
    DArr<long long> perm;
    DArr<float> loss;
    DArr<int> err;
    std::string msg;
};

static fcs_status mlp_err(fcs_mlp* m, fcs_status s, const std::string& what) {
    if (m) m->msg = what;
    return s;
}

#define MCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return mlp_err(mlp, FCS_ERR_CUDA, std::string(#call) + ": " +  \
                                                  cudaGetErrorString(e_));                     \
    } while (0)

static fcs_status check_device_err(fcs_mlp* mlp) {
    int h = 0;
    MCK(cudaMemcpyAsync(&h, mlp->err.p, sizeof(int), cudaMemcpyDeviceToHost, mlp->st));
    MCK(cudaStreamSynchronize(mlp->st));
    if (h) {
        cudaMemsetAsync(mlp->err.p, 0, sizeof(int), mlp->st);
        return mlp_err(mlp, FCS_ERR_CUDA, "tensor-core GEMM wait timed out (code " + std::to_string(h) + ")");
    }
    return FCS_OK;
}

// Publish the BF16 copies of every layer of member e (after set/init).
static fcs_status publish(fcs_mlp* mlp, int e) {
    Member& M = mlp->mem[e];
    for (size_t l = 0; l < mlp->L.size(); l++) {
        const Layer& y = mlp->L[l];
        adam_publish_kernel<<<blocks_for((long long)y.out * y.in + y.out, 256), 256, 0, mlp->st>>>(
            y.out, y.in, y.kPad, y.nPad, M.params.p + y.wOff, M.params.p + y.bOff, nullptr, nullptr, nullptr, nullptr,
            nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, M.W[l].p, M.WT[l].p);
        MCK(cudaGetLastError());
    }
    return FCS_OK;
}

static fcs_status ensure_acts(fcs_mlp* mlp, int64_t rows, bool training) {
    const int w = mlp->sh.width, k0 = mlp->L.front().kPad, no = mlp->L.back().nPad;
    const size_t r = (size_t)round_up((int)rows, 128);
    MCK(mlp->X.ensure(r * k0));
    MCK(mlp->Out.ensure(r * no));
    const int depth = mlp->sh.depth;
    mlp->Z.resize(depth);
    mlp->H.resize(depth);
    mlp->HT.resize(depth);
    if (!training) {
        // inference: two ping-pong hidden buffers
        MCK(mlp->H[0].ensure(r * w));
        if (depth > 1) MCK(mlp->H[1].ensure(r * w));
        return FCS_OK;
    }
    MCK(mlp->XT.ensure(r * k0));
    MCK(mlp->dOut.ensure(r * no));
    MCK(mlp->dOutT.ensure(r * no));
    MCK(mlp->dZT.ensure(r * w));
    MCK(mlp->dZ[0].ensure(r * w));
    MCK(mlp->dZ[1].ensure(r * w));
    for (int l = 0; l < depth; l++) {
        MCK(mlp->Z[l].ensure(r * w));
        MCK(mlp->H[l].ensure(r * w));
        MCK(mlp->HT[l].ensure(r * w));
    }
    return FCS_OK;
}

static GemmArgs base_args(fcs_mlp* mlp) {
    GemmArgs a{};
    a.err = mlp->err.p;
    return a;
}

// Forward pass of member e over the packed input mlp->X ([n][kPad0]).
// training: stores Z, H, H^T of every hidden layer and the normalised output
// in mlp->Out; inference: ping-pong hidden buffers, output de-normalised into
// y (ld n_out).
static fcs_status forward_packed(fcs_mlp* mlp, int e, int n, bool training, float* y, cudaStream_t st) {
    Member& M = mlp->mem[e];
    const int depth = mlp->sh.depth, w = mlp->sh.width;
    const int ldT = round_up(n, 128);
    const bf16* A = mlp->X.p;
    int lda = mlp->L[0].kPad;
    for (int l = 0; l <= depth; l++) {
        const Layer& ly = mlp->L[l];
        GemmArgs a = base_args(mlp);
        a.bias = M.params.p + ly.bOff;
        if (l < depth) {
            a.mode = EPI_HIDDEN;
            bf16* h = training ? mlp->H[l].p : mlp->H[l & 1].p;
            a.h = h; a.ldh = w;
            if (training) {
                a.z = mlp->Z[l].p; a.ldz = w;
                a.t = mlp->HT[l].p; a.ldt = ldT;
            }
            a.nValid = ly.nPad;
            MCK(gemm(A, lda, M.W[l].p, ly.kPad, n, ly.nPad, ly.kPad, 1, a, st));
            A = h;
            lda = w;
        } else {
            a.mode = EPI_OUT;
            a.nValid = ly.out;  // padding columns of the training output are never read
            if (training) {
                a.f = mlp->Out.p; a.ldf = ly.nPad;
            } else {
                a.f = y; a.ldf = ly.out;
                a.outScale = mlp->outStd.p; a.outShift = mlp->outMean.p;
            }
            MCK(gemm(A, lda, M.W[l].p, ly.kPad, n, ly.nPad, ly.kPad, 1, a, st));
        }
    }
    return FCS_OK;
}

// Backward pass of member e after forward_packed(training) and the loss
// kernel: fills mlp->gW / mlp->gb (zeroed here).
static fcs_status backward(fcs_mlp* mlp, int e, int n) {
    Member& M = mlp->mem[e];
    cudaStream_t st = mlp->st;
    const int depth = mlp->sh.depth, w = mlp->sh.width;
    const int ldT = round_up(n, 128);
    MCK(cudaMemsetAsync(mlp->gW.p, 0, mlp->gW.n * sizeof(float), st));
    const int splits = std::max(1, n / 512);
    // output layer
    {
        const Layer& ly = mlp->L[depth];
        GemmArgs a = base_args(mlp);
        a.mode = EPI_WGRAD;
        a.f = mlp->gW.p + ly.gOff; a.ldf = ly.kPad; a.nValid = ly.kPad;
        MCK(gemm(mlp->dOutT.p, ldT, mlp->HT[depth - 1].p, ldT, ly.nPad, ly.kPad, n, splits, a, st));
        rowsum_kernel<<<ly.nPad, 256, 0, st>>>(ly.nPad, n, mlp->dOutT.p, ldT, mlp->gb.p + ly.gbOff);
        MCK(cudaGetLastError());
        GemmArgs d = base_args(mlp);
        d.mode = EPI_DGRAD;
        d.h = mlp->dZ[(depth - 1) & 1].p; d.ldh = w;
        d.z = mlp->Z[depth - 1].p; d.ldz = w;
        d.t = mlp->dZT.p; d.ldt = ldT;
        d.nValid = w;
        MCK(gemm(mlp->dOut.p, ly.nPad, M.WT[depth].p, ly.nPad, n, w, ly.nPad, 1, d, st));
    }
    for (int l = depth - 1; l >= 0; l--) {
        const Layer& ly = mlp->L[l];
        GemmArgs a = base_args(mlp);
        a.mode = EPI_WGRAD;
        a.f = mlp->gW.p + ly.gOff; a.ldf = ly.kPad; a.nValid = ly.kPad;
        const bf16* Bt = l > 0 ? mlp->HT[l - 1].p : mlp->XT.p;
        MCK(gemm(mlp->dZT.p, ldT, Bt, ldT, ly.nPad, ly.kPad, n, splits, a, st));
        rowsum_kernel<<<ly.nPad, 256, 0, st>>>(ly.nPad, n, mlp->dZT.p, ldT, mlp->gb.p + ly.gbOff);
        MCK(cudaGetLastError());
        if (l > 0) {
            GemmArgs d = base_args(mlp);
            d.mode = EPI_DGRAD;
            d.h = mlp->dZ[(l - 1) & 1].p; d.ldh = w;
            d.z = mlp->Z[l - 1].p; d.ldz = w;
            d.t = mlp->dZT.p; d.ldt = ldT;
            d.nValid = w;
            MCK(gemm(mlp->dZ[l & 1].p, w, M.WT[l].p, ly.nPad, n, w, ly.nPad, 1, d, st));
        }
    }
    return FCS_OK;
}

// ---- C ABI -------------------------------------------------------------------

extern "C" fcs_status fcs_mlp_default_train_options(fcs_mlp_train_options* o) {
    if (!o) return FCS_ERR_INVALID;
    o->epochs = 20;
    o->batch = 4096;
    o->lr = 1e-3;
    o->lr_final = 2e-5;
    o->beta1 = 0.9;
    o->beta2 = 0.999;
    o->eps = 1e-8;
    o->seed = 1;
    return FCS_OK;
}

extern "C" const char* fcs_mlp_last_error(const fcs_mlp* m) { return m ? m->msg.c_str() : "null mlp"; }

extern "C" fcs_status fcs_mlp_get_shape(const fcs_mlp* m, fcs_mlp_shape* s) {
    if (!m || !s) return FCS_ERR_INVALID;
    *s = m->sh;
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_param_count(const fcs_mlp* m, int64_t* c) {
    if (!m || !c) return FCS_ERR_INVALID;
    *c = m->P;
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_destroy(fcs_mlp* mlp) {
    if (!mlp) return FCS_OK;
    cudaSetDevice(mlp->device);
    if (mlp->st) cudaStreamSynchronize(mlp->st);
    for (auto& M : mlp->mem) {
        M.params.release(); M.m.release(); M.v.release();
        for (auto& b : M.W) b.release();
        for (auto& b : M.WT) b.release();
    }
    for (auto* b : {&mlp->inMean, &mlp->inRstd, &mlp->outMean, &mlp->outStd, &mlp->gW, &mlp->gb, &mlp->Out,
                    &mlp->xDev, &mlp->yDev, &mlp->tDev, &mlp->loss})
        b->release();
    for (auto* b : {&mlp->X, &mlp->XT, &mlp->dOut, &mlp->dOutT, &mlp->dZT, &mlp->dZ[0], &mlp->dZ[1]}) b->release();
    for (auto& b : mlp->Z) b.release();
    for (auto& b : mlp->H) b.release();
    for (auto& b : mlp->HT) b.release();
    mlp->perm.release();
    mlp->err.release();
    if (mlp->st) cudaStreamDestroy(mlp->st);
    delete mlp;
    return FCS_OK;
}

static fcs_status set_norm(fcs_mlp* mlp, const float* im, const float* is, const float* om, const float* os) {
    const int ni = mlp->sh.n_in, no = mlp->sh.n_out;
    mlp->hInMean.assign(ni, 0.f); mlp->hInStd.assign(ni, 1.f);
    mlp->hOutMean.assign(no, 0.f); mlp->hOutStd.assign(no, 1.f);
    for (int i = 0; i < ni; i++) {
        if (im) mlp->hInMean[i] = im[i];
        if (is) mlp->hInStd[i] = is[i];
        if (!(mlp->hInStd[i] > 0)) return mlp_err(mlp, FCS_ERR_INVALID, "in_std must be positive");
    }
    for (int i = 0; i < no; i++) {
        if (om) mlp->hOutMean[i] = om[i];
        if (os) mlp->hOutStd[i] = os[i];
        if (!(mlp->hOutStd[i] > 0)) return mlp_err(mlp, FCS_ERR_INVALID, "out_std must be positive");
    }
    std::vector<float> rstd(ni);
    for (int i = 0; i < ni; i++) rstd[i] = 1.f / mlp->hInStd[i];
    MCK(cudaMemcpy(mlp->inMean.p, mlp->hInMean.data(), ni * 4, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(mlp->inRstd.p, rstd.data(), ni * 4, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(mlp->outMean.p, mlp->hOutMean.data(), no * 4, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(mlp->outStd.p, mlp->hOutStd.data(), no * 4, cudaMemcpyHostToDevice));
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_create(fcs_mlp** out, int device, const fcs_mlp_shape* s, uint64_t seed) {
    if (!out || !s) return FCS_ERR_INVALID;
    *out = nullptr;
    if (s->n_in < 1 || s->n_in > 256 || s->n_out < 1 || s->n_out > 256 || s->width != 256 || s->depth < 1 ||
        s->depth > 8 || s->members < 1 || s->members > 8)
        return FCS_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return FCS_ERR_CUDA;
    fcs_mlp* mlp = new fcs_mlp();
    mlp->device = device;
    mlp->sh = *s;
    if (cudaStreamCreateWithFlags(&mlp->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete mlp;
        return FCS_ERR_CUDA;
    }
    size_t off = 0, goff = 0, gboff = 0;
    for (int l = 0; l <= s->depth; l++) {
        Layer y;
        y.in = l == 0 ? s->n_in : s->width;
        y.out = l == s->depth ? s->n_out : s->width;
        y.kPad = round_up(y.in, 128);  // the K of the forward is the N of the weight gradient
        y.nPad = round_up(y.out, 128);
        y.wOff = off; off += (size_t)y.in * y.out;
        y.bOff = off; off += y.out;
        y.gOff = goff; goff += (size_t)y.nPad * y.kPad;
        y.gbOff = gboff; gboff += y.nPad;
        mlp->L.push_back(y);
    }
    mlp->P = (int64_t)off;
    fcs_status st = FCS_OK;
    auto fail = [&](fcs_status code) {
        fcs_mlp_destroy(mlp);
        return code;
    };
    if (mlp->gW.ensure(goff) || mlp->gb.ensure(gboff) || mlp->err.ensure(1) || mlp->loss.ensure(1) ||
        mlp->inMean.ensure(s->n_in) || mlp->inRstd.ensure(s->n_in) || mlp->outMean.ensure(s->n_out) ||
        mlp->outStd.ensure(s->n_out))
        return fail(FCS_ERR_NOMEM);
    if ((st = set_norm(mlp, nullptr, nullptr, nullptr, nullptr)) != FCS_OK) return fail(st);
    mlp->mem.resize(s->members);
    std::vector<float> host(off);
    for (int e = 0; e < s->members; e++) {
        Member& M = mlp->mem[e];
        if (M.params.ensure(off) || M.m.ensure(off) || M.v.ensure(off)) return fail(FCS_ERR_NOMEM);
        M.W.resize(mlp->L.size());
        M.WT.resize(mlp->L.size());
        for (size_t l = 0; l < mlp->L.size(); l++) {
            const Layer& y = mlp->L[l];
            if (M.W[l].ensure((size_t)y.nPad * y.kPad) || M.WT[l].ensure((size_t)y.nPad * y.kPad))
                return fail(FCS_ERR_NOMEM);
        }
        // He initialisation; the output layer starts 10x smaller
        std::mt19937_64 rng(seed + (uint64_t)e);
        std::fill(host.begin(), host.end(), 0.f);
        for (size_t l = 0; l < mlp->L.size(); l++) {
            const Layer& y = mlp->L[l];
            double sd = std::sqrt(2.0 / y.in);
            if ((int)l == s->depth) sd *= 0.1;
            std::normal_distribution<double> nd(0.0, sd);
            for (size_t i = 0; i < (size_t)y.in * y.out; i++) host[y.wOff + i] = (float)nd(rng);
        }
        if (cudaMemcpy(M.params.p, host.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(FCS_ERR_CUDA);
        if ((st = publish(mlp, e)) != FCS_OK) return fail(st);
    }
    if (cudaStreamSynchronize(mlp->st) != cudaSuccess) return fail(FCS_ERR_CUDA);
    *out = mlp;
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_set_params(fcs_mlp* mlp, int32_t e, const float* params) {
    if (!mlp || !params || e < 0 || e >= mlp->sh.members) return mlp_err(mlp, FCS_ERR_INVALID, "bad member or params");
    cudaSetDevice(mlp->device);
    Member& M = mlp->mem[e];
    MCK(cudaMemcpyAsync(M.params.p, params, mlp->P * 4, cudaMemcpyHostToDevice, mlp->st));
    MCK(cudaMemsetAsync(M.m.p, 0, mlp->P * 4, mlp->st));
    MCK(cudaMemsetAsync(M.v.p, 0, mlp->P * 4, mlp->st));
    M.step = 0;
    fcs_status s = publish(mlp, e);
    if (s != FCS_OK) return s;
    MCK(cudaStreamSynchronize(mlp->st));
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_get_params(const fcs_mlp* cm, int32_t e, float* params) {
    fcs_mlp* mlp = const_cast<fcs_mlp*>(cm);
    if (!mlp || !params || e < 0 || e >= mlp->sh.members) return mlp_err(mlp, FCS_ERR_INVALID, "bad member or params");
    cudaSetDevice(mlp->device);
    MCK(cudaMemcpyAsync(params, mlp->mem[e].params.p, mlp->P * 4, cudaMemcpyDeviceToHost, mlp->st));
    MCK(cudaStreamSynchronize(mlp->st));
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_set_normalization(fcs_mlp* mlp, const float* im, const float* is, const float* om,
                                                const float* os) {
    if (!mlp) return FCS_ERR_INVALID;
    cudaSetDevice(mlp->device);
    return set_norm(mlp, im, is, om, os);
}

extern "C" fcs_status fcs_mlp_get_normalization(const fcs_mlp* m, float* im, float* is, float* om, float* os) {
    if (!m) return FCS_ERR_INVALID;
    if (im) std::copy(m->hInMean.begin(), m->hInMean.end(), im);
    if (is) std::copy(m->hInStd.begin(), m->hInStd.end(), is);
    if (om) std::copy(m->hOutMean.begin(), m->hOutMean.end(), om);
    if (os) std::copy(m->hOutStd.begin(), m->hOutStd.end(), os);
    return FCS_OK;
}

fcs_status fcs::mlp_forward_device(fcs_mlp* mlp, int member, int64_t n, const float* x, float* y, cudaStream_t st) {
    if (!mlp || member < 0 || member >= mlp->sh.members) return mlp_err(mlp, FCS_ERR_INVALID, "bad member");
    if (n <= 0) return FCS_OK;
    if (n > (1LL << 24)) return mlp_err(mlp, FCS_ERR_INVALID, "too many rows");
    fcs_status s = ensure_acts(mlp, n, false);
    if (s != FCS_OK) return s;
    const Layer& l0 = mlp->L[0];
    pack_input_kernel<<<blocks_for(n * l0.kPad, 256), 256, 0, st>>>((int)n, l0.in, l0.kPad, x, nullptr, 0,
                                                                     mlp->inMean.p, mlp->inRstd.p, mlp->X.p, nullptr, 0);
    MCK(cudaGetLastError());
    return forward_packed(mlp, member, (int)n, false, y, st);
}

fcs_status fcs::mlp_check_errors(fcs_mlp* mlp) { return check_device_err(mlp); }

int fcs::mlp_n_in(const fcs_mlp* mlp) { return mlp->sh.n_in; }
int fcs::mlp_n_out(const fcs_mlp* mlp) { return mlp->sh.n_out; }
int fcs::mlp_members(const fcs_mlp* mlp) { return mlp->sh.members; }
int fcs::mlp_device(const fcs_mlp* mlp) { return mlp->device; }
const char* fcs::mlp_message(const fcs_mlp* mlp) { return mlp->msg.c_str(); }

extern "C" fcs_status fcs_mlp_forward(fcs_mlp* mlp, int32_t e, int64_t n, const float* x, float* y, int32_t flags) {
    if (!mlp || !x || !y) return mlp_err(mlp, FCS_ERR_INVALID, "null argument");
    if (e < 0 || e >= mlp->sh.members) return mlp_err(mlp, FCS_ERR_INVALID, "bad member");
    if (n <= 0) return FCS_OK;
    cudaSetDevice(mlp->device);
    const float* dx = x;
    float* dy = y;
    if (!(flags & FCS_PTR_DEVICE)) {
        MCK(mlp->xDev.ensure((size_t)n * mlp->sh.n_in));
        MCK(mlp->yDev.ensure((size_t)n * mlp->sh.n_out));
        MCK(cudaMemcpyAsync(mlp->xDev.p, x, (size_t)n * mlp->sh.n_in * 4, cudaMemcpyHostToDevice, mlp->st));
        dx = mlp->xDev.p;
        dy = mlp->yDev.p;
    }
    fcs_status s = fcs::mlp_forward_device(mlp, e, n, dx, dy, mlp->st);
    if (s != FCS_OK) return s;
    if (!(flags & FCS_PTR_DEVICE))
        MCK(cudaMemcpyAsync(y, dy, (size_t)n * mlp->sh.n_out * 4, cudaMemcpyDeviceToHost, mlp->st));
    return check_device_err(mlp);
}

// One training-mode forward + loss + backward over rows perm[off .. off+n)
// of the device-resident samples (perm null: rows 0..n-1).
static fcs_status fwd_bwd(fcs_mlp* mlp, int e, int n, const float* x, const float* t, const long long* perm,
                          long long off) {
    cudaStream_t st = mlp->st;
    const Layer& l0 = mlp->L[0];
    const Layer& lo = mlp->L.back();
    const int ldT = round_up(n, 128);
    pack_input_kernel<<<blocks_for((long long)n * l0.kPad, 256), 256, 0, st>>>(
        n, l0.in, l0.kPad, x, perm, off, mlp->inMean.p, mlp->inRstd.p, mlp->X.p, mlp->XT.p, ldT);
    MCK(cudaGetLastError());
    fcs_status s = forward_packed(mlp, e, n, true, nullptr, st);
    if (s != FCS_OK) return s;
    loss_grad_kernel<<<blocks_for((long long)n * lo.nPad, 256), 256, 0, st>>>(
        n, lo.out, lo.nPad, mlp->Out.p, t, perm, off, mlp->outMean.p, mlp->outStd.p, mlp->dOut.p, mlp->dOutT.p, ldT,
        mlp->loss.p);
    MCK(cudaGetLastError());
    return backward(mlp, e, n);
}

extern "C" fcs_status fcs_mlp_gradients(fcs_mlp* mlp, int32_t e, int64_t n, const float* x, const float* target,
                                        float* loss, float* grads) {
    if (!mlp || !x || !target) return mlp_err(mlp, FCS_ERR_INVALID, "null argument");
    if (e < 0 || e >= mlp->sh.members) return mlp_err(mlp, FCS_ERR_INVALID, "bad member");
    if (n <= 0 || n % 128 || n > (1 << 20)) return mlp_err(mlp, FCS_ERR_INVALID, "n must be a positive multiple of 128");
    cudaSetDevice(mlp->device);
    fcs_status s = ensure_acts(mlp, n, true);
    if (s != FCS_OK) return s;
    MCK(mlp->xDev.ensure((size_t)n * mlp->sh.n_in));
    MCK(mlp->tDev.ensure((size_t)n * mlp->sh.n_out));
    MCK(cudaMemcpyAsync(mlp->xDev.p, x, (size_t)n * mlp->sh.n_in * 4, cudaMemcpyHostToDevice, mlp->st));
    MCK(cudaMemcpyAsync(mlp->tDev.p, target, (size_t)n * mlp->sh.n_out * 4, cudaMemcpyHostToDevice, mlp->st));
    MCK(cudaMemsetAsync(mlp->loss.p, 0, sizeof(float), mlp->st));
    if ((s = fwd_bwd(mlp, e, (int)n, mlp->xDev.p, mlp->tDev.p, nullptr, 0)) != FCS_OK) return s;
    if ((s = check_device_err(mlp)) != FCS_OK) return s;
    float l = 0;
    MCK(cudaMemcpy(&l, mlp->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = l / (float)(n * mlp->sh.n_out);
    if (grads) {
        std::vector<float> gW(mlp->gW.n), gb(mlp->gb.n);
        MCK(cudaMemcpy(gW.data(), mlp->gW.p, gW.size() * 4, cudaMemcpyDeviceToHost));
        MCK(cudaMemcpy(gb.data(), mlp->gb.p, gb.size() * 4, cudaMemcpyDeviceToHost));
        for (const Layer& y : mlp->L) {
            for (int o = 0; o < y.out; o++) {
                for (int i = 0; i < y.in; i++) grads[y.wOff + (size_t)o * y.in + i] = gW[y.gOff + (size_t)o * y.kPad + i];
                grads[y.bOff + o] = gb[y.gbOff + o];
            }
        }
    }
    return FCS_OK;
}

extern "C" fcs_status fcs_mlp_train(fcs_mlp* mlp, int64_t n, const float* x, const float* target,
                                    const fcs_mlp_train_options* po, float* epoch_loss) {
    if (!mlp || !x || !target) return mlp_err(mlp, FCS_ERR_INVALID, "null argument");
    fcs_mlp_train_options o;
    fcs_mlp_default_train_options(&o);
    if (po) o = *po;
    if (o.batch <= 0 || o.batch % 128 || o.epochs <= 0 || !(o.lr > 0))
        return mlp_err(mlp, FCS_ERR_INVALID, "batch must be a positive multiple of 128; epochs and lr positive");
    if (n < o.batch) return mlp_err(mlp, FCS_ERR_INVALID, "fewer samples than one batch");
    cudaSetDevice(mlp->device);
    cudaStream_t st = mlp->st;
    fcs_status s = ensure_acts(mlp, o.batch, true);
    if (s != FCS_OK) return s;
    MCK(mlp->xDev.ensure((size_t)n * mlp->sh.n_in));
    MCK(mlp->tDev.ensure((size_t)n * mlp->sh.n_out));
    MCK(mlp->perm.ensure((size_t)n));
    MCK(cudaMemcpyAsync(mlp->xDev.p, x, (size_t)n * mlp->sh.n_in * 4, cudaMemcpyHostToDevice, st));
    MCK(cudaMemcpyAsync(mlp->tDev.p, target, (size_t)n * mlp->sh.n_out * 4, cudaMemcpyHostToDevice, st));
    const long long steps = n / o.batch;
    const long long total = steps * o.epochs;
    std::vector<long long> perm(n);
    for (int e = 0; e < mlp->sh.members; e++) {
        Member& M = mlp->mem[e];
        std::mt19937_64 rng(o.seed + (uint64_t)e);
        long long k = 0;
        for (int ep = 0; ep < o.epochs; ep++) {
            for (long long i = 0; i < n; i++) perm[i] = i;
            std::shuffle(perm.begin(), perm.end(), rng);
            MCK(cudaMemcpyAsync(mlp->perm.p, perm.data(), n * sizeof(long long), cudaMemcpyHostToDevice, st));
            MCK(cudaMemsetAsync(mlp->loss.p, 0, sizeof(float), st));
            for (long long b = 0; b < steps; b++, k++) {
                if ((s = fwd_bwd(mlp, e, o.batch, mlp->xDev.p, mlp->tDev.p, mlp->perm.p, b * o.batch)) != FCS_OK)
                    return s;
                // cosine decay from lr to lr_final
                const double frac = total > 1 ? (double)k / (double)(total - 1) : 0.0;
                const double lr = o.lr_final + 0.5 * (o.lr - o.lr_final) * (1.0 + std::cos(M_PI * frac));
                M.step++;
                const float c1 = (float)(1.0 / (1.0 - std::pow(o.beta1, (double)M.step)));
                const float c2 = (float)(1.0 / (1.0 - std::pow(o.beta2, (double)M.step)));
                for (const Layer& y : mlp->L) {
                    adam_publish_kernel<<<blocks_for((long long)y.out * y.in + y.out, 256), 256, 0, st>>>(
                        y.out, y.in, y.kPad, y.nPad, M.params.p + y.wOff, M.params.p + y.bOff, M.m.p + y.wOff,
                        M.v.p + y.wOff, M.m.p + y.bOff, M.v.p + y.bOff, mlp->gW.p + y.gOff, mlp->gb.p + y.gbOff,
                        (float)lr, (float)o.beta1, (float)o.beta2, (float)o.eps, c1, c2,
                        M.W[&y - &mlp->L[0]].p, M.WT[&y - &mlp->L[0]].p);
                }
                MCK(cudaGetLastError());
            }
            float l = 0;
            MCK(cudaMemcpyAsync(&l, mlp->loss.p, sizeof(float), cudaMemcpyDeviceToHost, st));
            if ((s = check_device_err(mlp)) != FCS_OK) return s;
            if (epoch_loss) epoch_loss[(size_t)e * o.epochs + ep] = l / (float)((double)steps * o.batch * mlp->sh.n_out);
        }
    }
    return check_device_err(mlp);
}

// ---- files ---------------------------------------------------------------------

static const char kMagic[8] = {'F', 'C', 'S', 'M', 'L', 'P', '1', 0};

extern "C" fcs_status fcs_mlp_save(const fcs_mlp* cm, const char* path) {
    fcs_mlp* mlp = const_cast<fcs_mlp*>(cm);
    if (!mlp || !path) return FCS_ERR_INVALID;
    FILE* f = std::fopen(path, "wb");
    if (!f) return mlp_err(mlp, FCS_ERR_INVALID, std::string("cannot write ") + path);
    std::vector<float> p(mlp->P);
    bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&mlp->sh, sizeof(fcs_mlp_shape), 1, f) == 1;
    ok = ok && std::fwrite(mlp->hInMean.data(), 4, mlp->sh.n_in, f) == (size_t)mlp->sh.n_in;
    ok = ok && std::fwrite(mlp->hInStd.data(), 4, mlp->sh.n_in, f) == (size_t)mlp->sh.n_in;
    ok = ok && std::fwrite(mlp->hOutMean.data(), 4, mlp->sh.n_out, f) == (size_t)mlp->sh.n_out;
    ok = ok && std::fwrite(mlp->hOutStd.data(), 4, mlp->sh.n_out, f) == (size_t)mlp->sh.n_out;
    for (int e = 0; ok && e < mlp->sh.members; e++) {
        if (fcs_mlp_get_params(mlp, e, p.data()) != FCS_OK) ok = false;
        ok = ok && std::fwrite(p.data(), 4, p.size(), f) == p.size();
    }
    std::fclose(f);
    return ok ? FCS_OK : mlp_err(mlp, FCS_ERR_INVALID, "write failed");
}

extern "C" fcs_status fcs_mlp_load(fcs_mlp** out, int device, const char* path) {
    if (!out || !path) return FCS_ERR_INVALID;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return FCS_ERR_INVALID;
    char magic[8];
    fcs_mlp_shape sh;
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) || std::fread(&sh, sizeof(sh), 1, f) != 1) {
        std::fclose(f);
        return FCS_ERR_PARSE;
    }
    fcs_mlp* mlp = nullptr;
    fcs_status s = fcs_mlp_create(&mlp, device, &sh, 0);
    if (s != FCS_OK) {
        std::fclose(f);
        return s;
    }
    std::vector<float> im(sh.n_in), is(sh.n_in), om(sh.n_out), os(sh.n_out), p(mlp->P);
    bool ok = std::fread(im.data(), 4, sh.n_in, f) == (size_t)sh.n_in && std::fread(is.data(), 4, sh.n_in, f) == (size_t)sh.n_in &&
              std::fread(om.data(), 4, sh.n_out, f) == (size_t)sh.n_out && std::fread(os.data(), 4, sh.n_out, f) == (size_t)sh.n_out;
    ok = ok && set_norm(mlp, im.data(), is.data(), om.data(), os.data()) == FCS_OK;
    for (int e = 0; ok && e < sh.members; e++) {
        ok = std::fread(p.data(), 4, p.size(), f) == p.size() && fcs_mlp_set_params(mlp, e, p.data()) == FCS_OK;
    }
    std::fclose(f);
    if (!ok) {
        fcs_mlp_destroy(mlp);
        return FCS_ERR_PARSE;
    }
    *out = mlp;
    return FCS_OK;
}
