// Warm-start network: a BF16 MLP (inputs -> L hidden GELU layers -> outputs)
// trained and evaluated on the tensor cores with FP32 accumulation.
//
// Every layer product is one TN GEMM, C[M x N] = A[M x K] * B[N x K]^T, both
// operands K-contiguous in HBM.  The epilogues write activations both as
// [rows][features] and transposed, so the forward pass, the input-gradient
// GEMMs (A = dZ, B = W) and the weight-gradient GEMMs (A = dZ^T, B = H^T)
// are all the same TN kernel.  Tiles of 64 x 64 x 32 are staged in shared
// memory with cp.async (double buffered), read with ldmatrix and multiplied
// with mma.sync m16n8k16 (BF16 in, FP32 accumulate).  Weight gradients
// reduce over the batch with a deterministic split-K (partials, then a fixed
// order sum), so training is bit-reproducible.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"
#include "mlp_act.cuh"
#include "mlp_tc.h"
#include "rng.cuh"

using bf16 = __nv_bfloat16;

namespace sp {
namespace mlp {

constexpr int BM = 64, BN = 64, BK = 32, PITCH = BK + 8;  // 80-byte rows: ldmatrix conflict-free

enum Epi { EPI_F32 = 0, EPI_BIAS_F32 = 1, EPI_BIAS_GELU = 2, EPI_GELU_BWD = 3 };

struct GemmArgs {
    const bf16* A;
    int lda;
    const bf16* B;
    int ldb;
    int M, N, K;
    int k_split;       // K elements per blockIdx.z (multiple of BK)
    float* C32;        // EPI_F32: partial [z][M][ldc]; EPI_BIAS_F32: [M][ldc]
    int ldc;
    const float* bias;  // [N]
    bf16* Z;            // EPI_BIAS_GELU: pre-activation [M][ld]
    bf16* H;            // EPI_BIAS_GELU: activation [M][ld]; EPI_GELU_BWD: dZ [M][ld]
    bf16* Ht;           // transposed copy [N][ldt]
    const bf16* Zin;    // EPI_GELU_BWD: stored pre-activation [M][ld]
    int ld, ldt;
    int* tc_err = nullptr;  // non-null: run on the tensor cores (mlptc::gemm) where the shape allows
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t r[4], const bf16* p) {
    unsigned s = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(s));
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

using act::gelu;
using act::gelu_grad;

template <int EPI>
__global__ void __launch_bounds__(128) gemm_tn(GemmArgs g) {
    __shared__ __align__(16) bf16 sA[2][BM * PITCH];
    __shared__ __align__(16) bf16 sB[2][BN * PITCH];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kb = blockIdx.z * g.k_split;
    const int ke = min(g.K, kb + g.k_split);
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

    auto load = [&](int stage, int k0) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int c = tid + i * 128;
            const int r = c >> 2, kc = (c & 3) * 8;
            const int gk = k0 + kc;
            const int gr = m0 + r;
            const bool oka = gr < g.M && gk < ke;
            cp_async16(&sA[stage][r * PITCH + kc], oka ? (const void*)(g.A + (size_t)gr * g.lda + gk) : (const void*)g.A,
                       oka ? 16 : 0);
            const int gn = n0 + r;
            const bool okb = gn < g.N && gk < ke;
            cp_async16(&sB[stage][r * PITCH + kc], okb ? (const void*)(g.B + (size_t)gn * g.ldb + gk) : (const void*)g.B,
                       okb ? 16 : 0);
        }
        cp_async_commit();
    };

    const int nk = ke > kb ? (ke - kb + BK - 1) / BK : 0;
    if (nk > 0) load(0, kb);
    for (int t = 0; t < nk; ++t) {
        if (t + 1 < nk) {
            load((t + 1) & 1, kb + (t + 1) * BK);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const bf16* a = sA[t & 1];
        const bf16* b = sB[t & 1];
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) {
                const int row = wm * 32 + mi * 16 + (lane & 15);
                const int col = kk + (lane >> 4) * 8;
                ldmatrix_x4(af[mi], &a[row * PITCH + col]);
            }
#pragma unroll
            for (int nj = 0; nj < 2; ++nj) {
                const int nrow = wn * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3);
                const int col = kk + ((lane >> 3) & 1) * 8;
                uint32_t r[4];
                ldmatrix_x4(r, &b[nrow * PITCH + col]);
                bfr[nj * 2][0] = r[0];
                bfr[nj * 2][1] = r[1];
                bfr[nj * 2 + 1][0] = r[2];
                bfr[nj * 2 + 1][1] = r[3];
            }
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], af[mi], bfr[ni]);
        }
        __syncthreads();
    }

#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int row = m0 + wm * 32 + mi * 16 + (lane >> 2) + ((e >> 1) << 3);
                const int col = n0 + wn * 32 + ni * 8 + (lane & 3) * 2 + (e & 1);
                if (row >= g.M || col >= g.N) continue;
                const float v = acc[mi][ni][e];
                if (EPI == EPI_F32) {
                    g.C32[((size_t)blockIdx.z * g.M + row) * g.ldc + col] = v;
                } else if (EPI == EPI_BIAS_F32) {
                    g.C32[(size_t)row * g.ldc + col] = v + g.bias[col];
                } else if (EPI == EPI_BIAS_GELU) {
                    const float z = v + g.bias[col];
                    const float h = gelu(z);
                    g.Z[(size_t)row * g.ld + col] = __float2bfloat16(z);
                    g.H[(size_t)row * g.ld + col] = __float2bfloat16(h);
                    g.Ht[(size_t)col * g.ldt + row] = __float2bfloat16(h);
                } else {
                    const float z = __bfloat162float(g.Zin[(size_t)row * g.ld + col]);
                    const bf16 d = __float2bfloat16(v * gelu_grad(z));
                    g.H[(size_t)row * g.ld + col] = d;
                    g.Ht[(size_t)col * g.ldt + row] = d;
                }
            }
}

template <int EPI>
cudaError_t gemm(const GemmArgs& g, int splits, cudaStream_t st) {
    if (g.tc_err) {
        static_assert(EPI_F32 == mlptc::kEpiF32 && EPI_BIAS_F32 == mlptc::kEpiBiasF32 &&
                          EPI_BIAS_GELU == mlptc::kEpiBiasGelu && EPI_GELU_BWD == mlptc::kEpiGeluBwd,
                      "epilogue codes");
        mlptc::GemmTcArgs t{g.A, g.lda, g.B, g.ldb, g.M, g.N, g.K, g.k_split, g.C32, g.ldc, g.bias,
                            g.Z, g.H, g.Ht, g.Zin, g.ld, g.ldt, EPI, g.tc_err, 0};
        if (mlptc::gemm_supported(t)) return mlptc::gemm(t, splits, st);
    }
    dim3 grid((g.M + BM - 1) / BM, (g.N + BN - 1) / BN, splits);
    gemm_tn<EPI><<<grid, 128, 0, st>>>(g);
    return cudaGetLastError();
}

// Sum split-K partials in split order: out[m][n] = sum_z part[z][m][n].
__global__ void splitk_reduce(const float* __restrict__ part, int splits, int count, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[(size_t)z * count + i];
    out[i] = s;
}

// Bias gradient: db[n] = sum over rows of dZ[row][n], in a fixed order: block
// (x, y) sums rows [y chunk, (y + 1) chunk) of columns 32x.. into part[y][n]
// (eight row lanes, then the lanes in order); bias_grad_final adds the
// chunks in order.  kBiasChunks chunks keep the whole GPU busy.
constexpr int kBiasChunks = 64;

__global__ void bias_grad(const bf16* __restrict__ d, int rows, int cols, int ld, float* __restrict__ part) {
    __shared__ float sh[8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int col = blockIdx.x * 32 + tx;
    const int chunk = (rows + gridDim.y - 1) / gridDim.y;
    const int r0 = blockIdx.y * chunk, r1 = min(rows, r0 + chunk);
    float s = 0.f;
    if (col < cols)
        for (int r = r0 + ty; r < r1; r += 8) s += __bfloat162float(d[(size_t)r * ld + col]);
    sh[ty][tx] = s;
    __syncthreads();
    if (ty == 0 && col < cols) {
        float t = 0.f;
        for (int k = 0; k < 8; ++k) t += sh[k][tx];
        part[(size_t)blockIdx.y * cols + col] = t;
    }
}

__global__ void bias_grad_final(const float* __restrict__ part, int chunks, int cols, float* __restrict__ db) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= cols) return;
    float t = 0.f;
    for (int y = 0; y < chunks; ++y) t += part[(size_t)y * cols + col];
    db[col] = t;
}

// Mean-squared-error gradient of the output layer (first n_real columns),
// written as dY [rows][ldy] and dY^T [ldy][rows]; accumulates the loss.
__global__ void mse_grad(const float* __restrict__ y, const float* __restrict__ t, int rows, int n_real, int ldy,
                         int ldt_in, bf16* __restrict__ dy, bf16* __restrict__ dyt, float* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < rows * ldy) {
        const int r = i / ldy, c = i % ldy;
        float g = 0.f;
        if (c < n_real) {
            const float diff = y[(size_t)r * ldy + c] - t[(size_t)r * ldt_in + c];
            l = diff * diff;
            g = 2.0f * diff / (float)(rows * n_real);
        }
        const bf16 gb = __float2bfloat16(g);
        dy[(size_t)r * ldy + c] = gb;
        dyt[(size_t)c * rows + r] = gb;
    }
    // warp reduction of the loss, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l / (float)(rows * n_real));
}

// Adam on FP32 master weights Wt [out][in] (+ bias), refreshing the BF16
// copies Wt (same layout) and W [in][out].  step is read from the device.
struct AdamArgs {
    float* w;
    float* m;
    float* v;
    const float* g;
    int count;       // elements of this tensor
    int rows, cols;  // for weights (Wt[rows][cols]); rows = 0 for a bias
    bf16* wt_bf;
    bf16* w_bf;
    float lr0, lr_min, beta1, beta2, eps;
    int total_steps;
    const int* step;
};

__global__ void adam(AdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    const int t = *a.step + 1;
    const float prog = fminf(1.0f, (float)(t - 1) / (float)max(a.total_steps, 1));
    const float lr = a.lr_min + 0.5f * (a.lr0 - a.lr_min) * (1.0f + cospif(prog));
    const float g = a.g[i];
    const float m = a.beta1 * a.m[i] + (1.f - a.beta1) * g;
    const float v = a.beta2 * a.v[i] + (1.f - a.beta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    const float mh = m / (1.f - powf(a.beta1, (float)t));
    const float vh = v / (1.f - powf(a.beta2, (float)t));
    const float w = a.w[i] - lr * mh / (sqrtf(vh) + a.eps);
    a.w[i] = w;
    if (a.rows > 0) {
        const int r = i / a.cols, c = i % a.cols;
        a.wt_bf[i] = __float2bfloat16(w);
        a.w_bf[(size_t)c * a.rows + r] = __float2bfloat16(w);
    }
}

__global__ void bump(int* step) { *step += 1; }

// BF16 copies of one weight tensor (after init or a host upload).
__global__ void refresh_bf16(const float* w, int rows, int cols, bf16* wt_bf, bf16* w_bf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int r = i / cols, c = i % cols;
    wt_bf[i] = __float2bfloat16(w[i]);
    w_bf[(size_t)c * rows + r] = __float2bfloat16(w[i]);
}

// FP32 inputs [rows][n_in] -> BF16 X [rows_pad][kin] and X^T [kin][rows_pad],
// zero in the padding.
__global__ void pack_inputs(const float* __restrict__ x, int rows, int rows_pad, int n_in, int kin,
                            bf16* __restrict__ X, bf16* __restrict__ Xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows_pad * kin) return;
    const int r = i / kin, c = i % kin;
    const float v = (r < rows && c < n_in) ? x[(size_t)r * n_in + c] : 0.f;
    const bf16 b = __float2bfloat16(v);
    X[i] = b;
    if (Xt) Xt[(size_t)c * rows_pad + r] = b;
}

// Inputs of the warm-start path: circuit parameters (SoA [slot][sample]) ->
// normalised BF16 X [rows_pad][kin].
__global__ void pack_params(const double* __restrict__ params_soa, size_t stride, int rows, int rows_pad,
                            const int* __restrict__ slots, const float* __restrict__ mean,
                            const float* __restrict__ scale, int n_in, int kin, bf16* __restrict__ X) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows_pad * kin) return;
    const int r = i / kin, c = i % kin;
    float v = 0.f;
    if (r < rows && c < n_in) v = (float)((params_soa[(size_t)slots[c] * stride + r] - (double)mean[c]) / (double)scale[c]);
    X[i] = __float2bfloat16(v);
}

// Outputs -> FP64 warm start x0 [rows][n_out] = mean + scale * y (+ linear term).
__global__ void unpack_outputs(const float* __restrict__ y, int rows, int ldy, int n_out, const float* __restrict__ mean,
                               const float* __restrict__ scale, double* __restrict__ x0, const double* __restrict__ lin,
                               const double* __restrict__ params_soa, size_t stride, const int* __restrict__ slots,
                               const float* __restrict__ in_mean, int n_in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * n_out) return;
    const int r = i / n_out, c = i % n_out;
    double x = (double)mean[c] + (double)scale[c] * (double)y[(size_t)r * ldy + c];
    if (lin)
        for (int j = 0; j < n_in; ++j)
            x += lin[c * n_in + j] * (params_soa[(size_t)slots[j] * stride + r] - (double)in_mean[j]);
    x0[i] = x;
}

// Deterministic He-uniform initialisation from the hash RNG.
__global__ void init_weights(float* w, int rows, int cols, int real_rows, int real_cols, float bound, uint64_t seed,
                             uint32_t tensor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int r = i / cols, c = i % cols;
    float v = 0.f;
    if (r < real_rows && c < real_cols) {
        uint64_t h = splitmix64(seed ^ ((uint64_t)tensor << 40) ^ (uint64_t)i);
        const double u = (double)(h >> 11) * 1.1102230246251565e-16;
        v = (float)((2.0 * u - 1.0) * bound);
    }
    w[i] = v;
}

__host__ __device__ inline int pad32(int x) { return (x + 31) & ~31; }

// Fused inference of the warm-start path: one CTA of 256 threads runs a tile
// of 64 samples through every layer.  Activations stay in shared memory
// (BF16, two ping-pong buffers); each layer's weights stream in 32-wide K
// chunks with cp.async (double buffered); warp w owns output columns
// [32w, 32w + 32) and all 64 rows (4 x 4 m16n8k16 tiles, FP32 accumulators).
// The output adds the FP64 linear term:
//   x0[k] = out_mean[k] + out_scale[k] * y[k] + sum_j lin[k][j] * (p_j - in_mean[j]).
constexpr int FT = 64;             // samples per CTA
constexpr int FH = 256;            // widest layer supported by the fused path
constexpr int APITCH = FH + 8;     // activation row pitch (elements)
constexpr int WPITCH = 40;         // weight chunk row pitch (elements)

struct FusedArgs {
    const double* params_soa;
    size_t stride;
    int rows;
    const int* slots;
    const float* io;      // in_mean[n_in], in_scale[n_in], out_mean[n_out], out_scale[n_out]
    const float* lin;     // [n_out][n_in] or nullptr (FP32: the warm start needs ~1e-3 relative)
    int n_in, n_out, kin, kout, H, L;
    const bf16* wt;       // per layer at woff[l]
    const float* params;  // biases at boff[l]
    int woff[9], boff[9];
    double* x0;
};

__global__ void __launch_bounds__(256) mlp_infer_fused(FusedArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    bf16* act0 = reinterpret_cast<bf16*>(fsm);
    bf16* act1 = act0 + FT * APITCH;
    bf16* wbuf = act1 + FT * APITCH;  // 2 x [FH][WPITCH]
    float* pc = reinterpret_cast<float*>(wbuf + 2 * FH * WPITCH);  // [FT][n_in] centred inputs
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = blockIdx.x * FT;
    // inputs: centred parameters (FP32, kept for the linear term) and their
    // normalised BF16 copies act0[:, 0:kin]
    for (int i = tid; i < FT * a.kin; i += 256) {
        const int r = i / a.kin, c = i % a.kin;
        float v = 0.f;
        if (r0 + r < a.rows && c < a.n_in) {
            const float d = (float)(a.params_soa[(size_t)a.slots[c] * a.stride + r0 + r] - (double)a.io[c]);
            pc[r * a.n_in + c] = d;
            v = d / a.io[a.n_in + c];
        } else if (c < a.n_in) {
            pc[r * a.n_in + c] = 0.f;
        }
        act0[r * APITCH + c] = __float2bfloat16(v);
    }
    bf16* in = act0;
    bf16* out = act1;
    int K = a.kin;
    for (int l = 0; l < a.L; ++l) {
        const bool last = (l == a.L - 1);
        const int N = last ? a.kout : a.H;
        const bf16* W = a.wt + a.woff[l];
        const float* bias = a.params + a.boff[l];
        const bool active = warp * 32 < N;
        float acc[4][4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
        auto load = [&](int stage, int k0) {
            bf16* dst = wbuf + stage * FH * WPITCH;
            for (int c = tid; c < N * 4; c += 256) {
                const int r = c >> 2, kc = (c & 3) * 8;
                cp_async16(&dst[r * WPITCH + kc], W + (size_t)r * K + k0 + kc, 16);
            }
            cp_async_commit();
        };
        const int nk = K / 32;
        __syncthreads();  // previous layer's activations are complete
        load(0, 0);
        for (int t = 0; t < nk; ++t) {
            if (t + 1 < nk) {
                load((t + 1) & 1, (t + 1) * 32);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            const bf16* wb = wbuf + (t & 1) * FH * WPITCH;
            if (active) {
#pragma unroll
                for (int kk = 0; kk < 32; kk += 16) {
                    uint32_t af[4][4], bfr[4][2];
#pragma unroll
                    for (int mi = 0; mi < 4; ++mi)
                        ldmatrix_x4(af[mi], &in[(mi * 16 + (lane & 15)) * APITCH + t * 32 + kk + (lane >> 4) * 8]);
#pragma unroll
                    for (int nj = 0; nj < 2; ++nj) {
                        uint32_t r[4];
                        ldmatrix_x4(r, &wb[(warp * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3)) * WPITCH + kk +
                                           ((lane >> 3) & 1) * 8]);
                        bfr[nj * 2][0] = r[0];
                        bfr[nj * 2][1] = r[1];
                        bfr[nj * 2 + 1][0] = r[2];
                        bfr[nj * 2 + 1][1] = r[3];
                    }
#pragma unroll
                    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                        for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], af[mi], bfr[ni]);
                }
            }
            __syncthreads();
        }
        if (active) {
#pragma unroll
            for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni)
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int row = mi * 16 + (lane >> 2) + ((e >> 1) << 3);
                        const int col = warp * 32 + ni * 8 + (lane & 3) * 2 + (e & 1);
                        const float v = acc[mi][ni][e] + bias[col];
                        if (!last) {
                            out[row * APITCH + col] = __float2bfloat16(gelu(v));
                        } else if (col < a.n_out && r0 + row < a.rows) {
                            const int s = r0 + row;
                            float x = a.io[2 * a.n_in + col] + a.io[2 * a.n_in + a.n_out + col] * v;
                            if (a.lin)
                                for (int j = 0; j < a.n_in; ++j) x = fmaf(a.lin[col * a.n_in + j], pc[row * a.n_in + j], x);
                            a.x0[(size_t)s * a.n_out + col] = (double)x;
                        }
                    }
        }
        bf16* tmp = in;
        in = out;
        out = tmp;
        K = N;
    }
}

}  // namespace mlp
}  // namespace sp

using namespace sp;
using namespace sp::mlp;

// One BF16 MLP: n_in -> n_layers x n_hidden (GELU) -> n_out.
struct sp_mlp {
    sp_ctx* ctx = nullptr;
    sp_mlp_desc d{};
    int kin = 0, kout = 0, H = 0, L = 0;  // padded in/out, hidden, number of GEMM layers
    std::vector<int> rows, cols;          // layer l: Wt [rows[l]][cols[l]] = [out][in]
    std::vector<size_t> woff, boff;       // offsets into the flat FP32 parameter vector
    size_t nparams = 0;
    float* params = nullptr;  // FP32 master: per layer Wt then b
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* grads = nullptr;  // same layout
    bf16* wt_bf = nullptr;   // per layer Wt (same offsets as params' weights)
    bf16* w_bf = nullptr;    // per layer W (transposed)
    int* step = nullptr;
    // I/O of the warm-start path
    int* io_slots = nullptr;  // [n_in]
    std::vector<int> h_slots; // the same on the host
    std::vector<float> h_io;  // io on the host
    std::vector<float> h_lin; // lin_f32 on the host
    int max_slot = -1;        // largest input slot (checked against the circuit)
    double* lin = nullptr;    // linear term [n_out][n_in] of the warm start (as given)
    float* lin_f32 = nullptr; // the same in FP32 for the fused kernel
    bool has_lin = false;
    bool fused_ready = false;
    // tcgen05 inference (mlp_tc.cu): packed weight image, gathered biases
    int kernel_kind = SP_MLP_KERNEL_AUTO;
    int train_kind = SP_MLP_KERNEL_AUTO;  // GEMMs of training: tcgen05 where the shape allows, or mma.sync
    bool tc_dirty = true;     // weights changed since the image was packed
    void* tc_img = nullptr;
    float* tc_bias = nullptr;
    int* tc_err = nullptr;
    int num_sms = 0;
    float* io = nullptr;      // in_mean[n_in], in_scale[n_in], out_mean[n_out], out_scale[n_out]
    bool io_set = false;
    // activation workspace for `ws_rows` rows
    int ws_rows = 0;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    bf16 *X = nullptr, *Xt = nullptr;
    std::vector<bf16*> Z, Hb, Ht;  // per hidden layer
    float* Y = nullptr;
    bf16 *dY = nullptr, *dYt = nullptr, *dA = nullptr, *dB = nullptr, *dAt = nullptr, *dBt = nullptr;
    float* part = nullptr;  // split-K partials
    size_t part_elems = 0;
    float* loss = nullptr;
};

namespace sp {
bool tc_eligible(const sp_mlp* m);
}

namespace {

size_t a256m(size_t b) { return (b + 255) & ~size_t(255); }

int mlp_fail(sp_ctx* ctx, int code, const char* msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

constexpr int kSplitRows = 128;  // batch rows per split of a weight-gradient GEMM (one CTA each)
constexpr uint64_t kMaxRows = 1u << 22;  // keeps every element index of the workspace within int

int ensure_ws(sp_mlp* m, int rows) {
    const int rp = (rows + 63) & ~63;
    if (rp <= m->ws_rows) return SP_OK;
    const int Hd = m->H, nl = m->L - 1;
    size_t b = 0;
    auto take = [&](size_t bytes) {
        size_t o = b;
        b += a256m(bytes);
        return o;
    };
    size_t oX = take(2ull * rp * m->kin), oXt = take(2ull * rp * m->kin);
    std::vector<size_t> oZ(nl), oH(nl), oHt(nl);
    for (int l = 0; l < nl; ++l) {
        oZ[l] = take(2ull * rp * Hd);
        oH[l] = take(2ull * rp * Hd);
        oHt[l] = take(2ull * rp * Hd);
    }
    size_t oY = take(4ull * rp * m->kout), odY = take(2ull * rp * m->kout), odYt = take(2ull * rp * m->kout);
    size_t odA = take(2ull * rp * Hd), odB = take(2ull * rp * Hd), odAt = take(2ull * rp * Hd),
           odBt = take(2ull * rp * Hd);
    const int splits = (rp + kSplitRows - 1) / kSplitRows;
    size_t maxw = (size_t)Hd * std::max(Hd, std::max(m->kin, m->kout));
    size_t opart = take(4ull * splits * maxw);
    size_t oloss = take(256);
    // the callers hold the context's ordering guard: the old workspace is
    // freed in stream order after its last user
    const int rc = grow_buffer(m->ctx, &m->ws, &m->ws_bytes, b, "MLP workspace");
    if (rc != SP_OK) {
        m->ws_rows = 0;
        return rc;
    }
    char* p = (char*)m->ws;
    m->ws_rows = rp;
    m->X = (bf16*)(p + oX);
    m->Xt = (bf16*)(p + oXt);
    m->Z.resize(nl);
    m->Hb.resize(nl);
    m->Ht.resize(nl);
    for (int l = 0; l < nl; ++l) {
        m->Z[l] = (bf16*)(p + oZ[l]);
        m->Hb[l] = (bf16*)(p + oH[l]);
        m->Ht[l] = (bf16*)(p + oHt[l]);
    }
    m->Y = (float*)(p + oY);
    m->dY = (bf16*)(p + odY);
    m->dYt = (bf16*)(p + odYt);
    m->dA = (bf16*)(p + odA);
    m->dB = (bf16*)(p + odB);
    m->dAt = (bf16*)(p + odAt);
    m->dBt = (bf16*)(p + odBt);
    m->part = (float*)(p + opart);
    m->part_elems = splits * maxw;
    m->loss = (float*)(p + oloss);
    return SP_OK;
}

// Forward over rows already packed into m->X (rows_pad rows); Y = outputs.
// Error flag of the tcgen05 training GEMMs (an int inside the step block,
// zeroed at creation), or nullptr when training runs on mma.sync.
int* train_tc_err(const sp_mlp* m) {
    return m->train_kind == SP_MLP_KERNEL_MMA_SYNC ? nullptr : m->step + 16;
}

cudaError_t forward(sp_mlp* m, int rows_pad, bool keep, cudaStream_t st) {
    const int nl = m->L - 1;
    const bf16* in = m->X;
    int kin = m->kin;
    for (int l = 0; l < nl; ++l) {
        GemmArgs g{};
        g.tc_err = train_tc_err(m);
        g.A = in;
        g.lda = kin;
        g.B = m->wt_bf + m->woff[l];
        g.ldb = m->cols[l];
        g.M = rows_pad;
        g.N = m->rows[l];
        g.K = kin;
        g.k_split = pad32(kin);
        g.bias = m->params + m->boff[l];
        g.Z = m->Z[l];
        g.H = m->Hb[l];
        g.Ht = m->Ht[l];
        g.ld = m->H;
        g.ldt = rows_pad;
        cudaError_t e = gemm<EPI_BIAS_GELU>(g, 1, st);
        if (e != cudaSuccess) return e;
        in = m->Hb[l];
        kin = m->H;
        (void)keep;
    }
    GemmArgs g{};
    g.tc_err = train_tc_err(m);
    g.A = in;
    g.lda = kin;
    g.B = m->wt_bf + m->woff[nl];
    g.ldb = m->cols[nl];
    g.M = rows_pad;
    g.N = m->kout;
    g.K = kin;
    g.k_split = kin;
    g.C32 = m->Y;
    g.ldc = m->kout;
    g.bias = m->params + m->boff[nl];
    return gemm<EPI_BIAS_F32>(g, 1, st);
}

// Backward for the batch held in the workspace; writes m->grads.
cudaError_t backward(sp_mlp* m, int rows_pad, const float* targets, int ldt_in, cudaStream_t st) {
    const int nl = m->L - 1;
    cudaError_t e;
    {
        const int total = rows_pad * m->kout;
        mse_grad<<<(total + 255) / 256, 256, 0, st>>>(m->Y, targets, rows_pad, m->d.n_out, m->kout, ldt_in, m->dY,
                                                      m->dYt, m->loss);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const int splits = (rows_pad + kSplitRows - 1) / kSplitRows;
    const bf16* dcur = m->dY;    // dZ of the current layer [rows][width]
    const bf16* dcurT = m->dYt;  // transposed [width][rows]
    int width = m->kout;
    bool toggle = false;
    for (int l = nl; l >= 0; --l) {
        const bf16* inT = (l == 0) ? m->Xt : m->Ht[l - 1];
        const int in_w = (l == 0) ? m->kin : m->H;
        // weight gradient: dWt[out][in] = dZ^T [out][rows] * (H^T [in][rows])^T
        GemmArgs g{};
        g.tc_err = train_tc_err(m);
        g.A = dcurT;
        g.lda = rows_pad;
        g.B = inT;
        g.ldb = rows_pad;
        g.M = width;
        g.N = in_w;
        g.K = rows_pad;
        g.k_split = kSplitRows;
        g.C32 = m->part;
        g.ldc = in_w;
        if ((e = gemm<EPI_F32>(g, splits, st)) != cudaSuccess) return e;
        const int cnt = width * in_w;
        splitk_reduce<<<(cnt + 255) / 256, 256, 0, st>>>(m->part, splits, cnt, m->grads + m->woff[l]);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        {
            const int chunks = (int)std::max<size_t>(
                1, std::min<size_t>({(size_t)kBiasChunks, (size_t)rows_pad / 64, m->part_elems / (size_t)width}));
            bias_grad<<<dim3((width + 31) / 32, chunks), 256, 0, st>>>(dcur, rows_pad, width, width, m->part);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            bias_grad_final<<<(width + 127) / 128, 128, 0, st>>>(m->part, chunks, width, m->grads + m->boff[l]);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (l == 0) break;
        // input gradient through the GELU: dZ_{l-1} = (dZ_l * W_l) .* gelu'(Z_{l-1})
        bf16* dn = toggle ? m->dB : m->dA;
        bf16* dnT = toggle ? m->dBt : m->dAt;
        toggle = !toggle;
        GemmArgs h{};
        h.tc_err = train_tc_err(m);
        h.A = dcur;
        h.lda = width;
        h.B = m->w_bf + m->woff[l];  // W [in][out]
        h.ldb = width;
        h.M = rows_pad;
        h.N = in_w;
        h.K = width;
        h.k_split = pad32(width);
        h.Zin = m->Z[l - 1];
        h.H = dn;
        h.Ht = dnT;
        h.ld = m->H;
        h.ldt = rows_pad;
        if ((e = gemm<EPI_GELU_BWD>(h, 1, st)) != cudaSuccess) return e;
        dcur = dn;
        dcurT = dnT;
        width = m->H;
    }
    return cudaSuccess;
}

cudaError_t adam_step(sp_mlp* m, float lr, int total_steps, cudaStream_t st) {
    for (int l = 0; l < m->L; ++l) {
        AdamArgs a{};
        a.lr0 = lr;
        a.lr_min = lr * 0.01f;
        a.beta1 = 0.9f;
        a.beta2 = 0.999f;
        a.eps = 1e-8f;
        a.total_steps = total_steps;
        a.step = m->step;
        a.w = m->params + m->woff[l];
        a.m = m->adam_m + m->woff[l];
        a.v = m->adam_v + m->woff[l];
        a.g = m->grads + m->woff[l];
        a.count = m->rows[l] * m->cols[l];
        a.rows = m->rows[l];
        a.cols = m->cols[l];
        a.wt_bf = m->wt_bf + m->woff[l];
        a.w_bf = m->w_bf + m->woff[l];
        adam<<<(a.count + 255) / 256, 256, 0, st>>>(a);
        AdamArgs b = a;
        b.w = m->params + m->boff[l];
        b.m = m->adam_m + m->boff[l];
        b.v = m->adam_v + m->boff[l];
        b.g = m->grads + m->boff[l];
        b.count = m->rows[l];
        b.rows = 0;
        adam<<<(b.count + 255) / 256, 256, 0, st>>>(b);
    }
    bump<<<1, 1, 0, st>>>(m->step);
    return cudaGetLastError();
}

cudaError_t refresh_all(sp_mlp* m, cudaStream_t st) {
    for (int l = 0; l < m->L; ++l) {
        const int cnt = m->rows[l] * m->cols[l];
        refresh_bf16<<<(cnt + 255) / 256, 256, 0, st>>>(m->params + m->woff[l], m->rows[l], m->cols[l],
                                                        m->wt_bf + m->woff[l], m->w_bf + m->woff[l]);
    }
    return cudaGetLastError();
}

}  // namespace

extern "C" {

int sp_mlp_create(sp_ctx* ctx, const sp_mlp_desc* d, sp_mlp** out) {
    if (!ctx || !d || !out) return SP_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (d->n_in < 1 || d->n_in > 64 || d->n_out < 1 || d->n_out > 64 || d->n_hidden < 32 || d->n_hidden > 1024 ||
        d->n_hidden % 32 || d->n_layers < 1 || d->n_layers > 8)
        return mlp_fail(ctx, SP_ERR_INVALID_DIMENSION, "unsupported MLP shape");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    sp_mlp* m = new sp_mlp();
    m->ctx = ctx;
    m->d = *d;
    m->kin = pad32(d->n_in);
    m->kout = pad32(d->n_out);
    m->H = d->n_hidden;
    m->L = d->n_layers + 1;
    size_t off = 0;
    for (int l = 0; l < m->L; ++l) {
        const int in = (l == 0) ? m->kin : m->H;
        const int outw = (l == m->L - 1) ? m->kout : m->H;
        m->rows.push_back(outw);
        m->cols.push_back(in);
        m->woff.push_back(off);
        off += (size_t)outw * in;
        m->boff.push_back(off);
        off += outw;
    }
    m->nparams = off;
    const size_t bytes = off * 4;
    cudaError_t e = cudaMalloc(&m->params, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&m->adam_m, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&m->adam_v, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&m->grads, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&m->wt_bf, off * 2);
    if (e == cudaSuccess) e = cudaMalloc(&m->w_bf, off * 2);
    if (e == cudaSuccess) e = cudaMalloc(&m->step, 256);
    if (e == cudaSuccess) e = cudaMalloc(&m->io_slots, 4 * 64);
    if (e == cudaSuccess) e = cudaMalloc(&m->io, 4 * 256);
    if (e != cudaSuccess) {
        delete m;
        return mlp_fail(ctx, SP_ERR_MEMORY_ALLOC, "MLP allocation");
    }
    cudaMemset(m->params, 0, bytes);
    cudaMemset(m->adam_m, 0, bytes);
    cudaMemset(m->adam_v, 0, bytes);
    cudaMemset(m->grads, 0, bytes);
    cudaMemset(m->step, 0, 256);
    for (int l = 0; l < m->L; ++l) {
        const int real_in = (l == 0) ? d->n_in : m->H;
        const int real_out = (l == m->L - 1) ? d->n_out : m->H;
        const int cnt = m->rows[l] * m->cols[l];
        const float bound = sqrtf(6.0f / (float)real_in);
        init_weights<<<(cnt + 255) / 256, 256>>>(m->params + m->woff[l], m->rows[l], m->cols[l], real_out, real_in,
                                                bound, d->init_seed, (uint32_t)l);
    }
    e = refresh_all(m, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        delete m;
        return mlp_fail(ctx, SP_ERR_BACKEND, "MLP initialisation");
    }
    *out = m;
    return SP_OK;
}

int sp_mlp_destroy(sp_mlp* m) {
    if (!m) return SP_OK;
    cudaSetDevice(m->ctx->device);
    cudaDeviceSynchronize();
    if (m->ws) {  // from the stream-ordered allocator
        cudaFreeAsync(m->ws, m->ctx->stream);
        cudaStreamSynchronize(m->ctx->stream);
    }
    for (void* p : {(void*)m->params, (void*)m->adam_m, (void*)m->adam_v, (void*)m->grads, (void*)m->wt_bf,
                    (void*)m->w_bf, (void*)m->step, (void*)m->io_slots, (void*)m->io, (void*)m->lin,
                    (void*)m->lin_f32, m->tc_img, (void*)m->tc_bias, (void*)m->tc_err})
        if (p) cudaFree(p);
    delete m;
    return SP_OK;
}

int sp_mlp_num_params(const sp_mlp* m) { return m ? (int)m->nparams : 0; }

int sp_mlp_get_params(sp_mlp* m, float* host) {
    if (!m || !host) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    return cudaMemcpy(host, m->params, m->nparams * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? SP_OK : SP_ERR_TRANSFER;
}

int sp_mlp_set_params(sp_mlp* m, const float* host) {
    if (!m || !host) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    if (cudaMemcpy(m->params, host, m->nparams * 4, cudaMemcpyHostToDevice) != cudaSuccess) return SP_ERR_TRANSFER;
    cudaMemset(m->adam_m, 0, m->nparams * 4);
    cudaMemset(m->adam_v, 0, m->nparams * 4);
    cudaMemset(m->step, 0, 4);
    m->tc_dirty = true;
    if (refresh_all(m, 0) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return SP_ERR_BACKEND;
    return SP_OK;
}

int sp_mlp_set_io(sp_mlp* m, const int32_t* in_slots, const float* in_mean, const float* in_scale,
                  const float* out_mean, const float* out_scale) {
    if (!m || !in_slots || !in_mean || !in_scale || !out_mean || !out_scale) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    std::vector<float> io(2 * m->d.n_in + 2 * m->d.n_out);
    std::memcpy(io.data(), in_mean, 4 * m->d.n_in);
    std::memcpy(io.data() + m->d.n_in, in_scale, 4 * m->d.n_in);
    std::memcpy(io.data() + 2 * m->d.n_in, out_mean, 4 * m->d.n_out);
    std::memcpy(io.data() + 2 * m->d.n_in + m->d.n_out, out_scale, 4 * m->d.n_out);
    m->max_slot = -1;
    for (int j = 0; j < m->d.n_in; ++j) {
        if (in_slots[j] < 0) return mlp_fail(m->ctx, SP_ERR_INVALID_ARGUMENT, "negative input slot");
        m->max_slot = std::max(m->max_slot, (int)in_slots[j]);
    }
    m->h_slots.assign(in_slots, in_slots + m->d.n_in);
    m->h_io = io;
    if (cudaMemcpy(m->io, io.data(), 4 * io.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->io_slots, in_slots, 4 * m->d.n_in, cudaMemcpyHostToDevice) != cudaSuccess)
        return SP_ERR_TRANSFER;
    m->io_set = true;
    return SP_OK;
}

int sp_mlp_forward_device(sp_mlp* m, const float* d_x, uint64_t rows, float* d_y, void* stream) {
    if (!m || !d_x || !d_y) return SP_ERR_INVALID_ARGUMENT;
    if (rows == 0) return SP_OK;
    if (rows > kMaxRows) {
        char msg[96];
        snprintf(msg, sizeof msg, "Batch size %llu exceeds maximum %llu", (unsigned long long)rows,
                 (unsigned long long)kMaxRows);
        return mlp_fail(m->ctx, SP_ERR_BATCH_TOO_LARGE, msg);
    }
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(m->ctx, st);  // orders workspace reuse and growth after earlier users
    if (ensure_ws(m, (int)rows) != SP_OK) return mlp_fail(m->ctx, SP_ERR_MEMORY_ALLOC, "MLP workspace");
    const int rp = ((int)rows + 63) & ~63;
    ProfScope prof(m->ctx, "mlp_forward", st);
    pack_inputs<<<(rp * m->kin + 255) / 256, 256, 0, st>>>(d_x, (int)rows, rp, m->d.n_in, m->kin, m->X, nullptr);
    if (forward(m, rp, false, st) != cudaSuccess) return mlp_fail(m->ctx, SP_ERR_BACKEND, "MLP forward");
    // copy out the real columns
    if (cudaMemcpy2DAsync(d_y, 4 * m->d.n_out, m->Y, 4 * m->kout, 4 * m->d.n_out, rows, cudaMemcpyDeviceToDevice,
                          st) != cudaSuccess)
        return mlp_fail(m->ctx, SP_ERR_BACKEND, "MLP output copy");
    return SP_OK;
}

int sp_mlp_gradients_device(sp_mlp* m, const float* d_x, const float* d_t, uint64_t rows, float* d_grads,
                            float* d_loss, void* stream) {
    if (!m || !d_x || !d_t || !d_grads) return SP_ERR_INVALID_ARGUMENT;
    if (rows == 0 || rows > kMaxRows) return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "bad row count");
    if (rows % 64) return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "gradient batches are multiples of 64 rows");
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(m->ctx, st);  // orders workspace reuse and growth after earlier users
    if (ensure_ws(m, (int)rows) != SP_OK) return mlp_fail(m->ctx, SP_ERR_MEMORY_ALLOC, "MLP workspace");
    const int rp = (int)rows;
    pack_inputs<<<(rp * m->kin + 255) / 256, 256, 0, st>>>(d_x, rp, rp, m->d.n_in, m->kin, m->X, m->Xt);
    cudaMemsetAsync(m->loss, 0, 4, st);
    if (forward(m, rp, true, st) != cudaSuccess || backward(m, rp, d_t, m->d.n_out, st) != cudaSuccess)
        return mlp_fail(m->ctx, SP_ERR_BACKEND, "MLP gradients");
    cudaMemcpyAsync(d_grads, m->grads, m->nparams * 4, cudaMemcpyDeviceToDevice, st);
    if (d_loss) cudaMemcpyAsync(d_loss, m->loss, 4, cudaMemcpyDeviceToDevice, st);
    return cudaGetLastError() == cudaSuccess ? SP_OK : SP_ERR_BACKEND;
}

int sp_mlp_train_device(sp_mlp* m, const float* d_x, const float* d_t, uint64_t rows, int batch, int epochs,
                        float lr, float* d_epoch_loss, void* stream) {
    if (!m || !d_x || !d_t) return SP_ERR_INVALID_ARGUMENT;
    if (batch < 64 || batch % 64 || (uint64_t)batch > rows || (uint64_t)batch > kMaxRows || epochs < 1)
        return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "batch must be a multiple of 64, <= rows");
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(m->ctx, st);  // orders workspace reuse and growth after earlier users
    if (ensure_ws(m, batch) != SP_OK) return mlp_fail(m->ctx, SP_ERR_MEMORY_ALLOC, "MLP workspace");
    const uint64_t steps_per_epoch = rows / batch;
    const int total = (int)(steps_per_epoch * epochs);
    ProfScope prof(m->ctx, "mlp_train", st);
    m->tc_dirty = true;
    for (int ep = 0; ep < epochs; ++ep) {
        cudaMemsetAsync(m->loss, 0, 4, st);
        for (uint64_t s = 0; s < steps_per_epoch; ++s) {
            const float* xb = d_x + s * batch * m->d.n_in;
            const float* tb = d_t + s * batch * m->d.n_out;
            pack_inputs<<<(batch * m->kin + 255) / 256, 256, 0, st>>>(xb, batch, batch, m->d.n_in, m->kin, m->X,
                                                                      m->Xt);
            if (forward(m, batch, true, st) != cudaSuccess || backward(m, batch, tb, m->d.n_out, st) != cudaSuccess ||
                adam_step(m, lr, total, st) != cudaSuccess)
                return mlp_fail(m->ctx, SP_ERR_BACKEND, "MLP training step");
        }
        if (d_epoch_loss) {
            // the loss accumulator holds the sum over this epoch's batches of the batch mean
            cudaMemcpyAsync(d_epoch_loss + ep, m->loss, 4, cudaMemcpyDeviceToDevice, st);
        }
    }
    return cudaGetLastError() == cudaSuccess ? SP_OK : SP_ERR_BACKEND;
}

}  // extern "C"

extern "C" int sp_mlp_set_linear(sp_mlp* m, const double* lin) {
    if (!m) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    if (!lin) {
        m->has_lin = false;
        return SP_OK;
    }
    const size_t cnt = (size_t)m->d.n_out * m->d.n_in;
    if (!m->lin && cudaMalloc(&m->lin, sizeof(double) * cnt) != cudaSuccess)
        return mlp_fail(m->ctx, SP_ERR_MEMORY_ALLOC, "linear term");
    if (!m->lin_f32 && cudaMalloc(&m->lin_f32, sizeof(float) * cnt) != cudaSuccess)
        return mlp_fail(m->ctx, SP_ERR_MEMORY_ALLOC, "linear term");
    std::vector<float> f(lin, lin + cnt);
    if (cudaMemcpy(m->lin, lin, sizeof(double) * cnt, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->lin_f32, f.data(), sizeof(float) * cnt, cudaMemcpyHostToDevice) != cudaSuccess)
        return SP_ERR_TRANSFER;
    m->has_lin = true;
    m->h_lin = f;
    return SP_OK;
}

extern "C" int sp_mlp_set_inference_kernel(sp_mlp* m, int kind) {
    if (!m || kind < SP_MLP_KERNEL_AUTO || kind > SP_MLP_KERNEL_LINEAR) return SP_ERR_INVALID_ARGUMENT;
    if (kind == SP_MLP_KERNEL_LINEAR && !m->has_lin)
        return mlp_fail(m->ctx, SP_ERR_INVALID_ARGUMENT, "the linear warm start needs sp_mlp_set_linear first");
    if (kind == SP_MLP_KERNEL_TCGEN05 && !sp::tc_eligible(m))
        return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION,
                        "tcgen05 inference needs n_in <= 32, n_out <= 32, hidden 64, 128 or 256, 1..4 hidden layers");
    if (kind == SP_MLP_KERNEL_MMA_SYNC && !(m->H <= FH && m->L <= 9))
        return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "the fused mma.sync kernel needs hidden <= 256");
    std::lock_guard<std::mutex> g(m->ctx->mu);
    m->kernel_kind = kind;
    return SP_OK;
}

extern "C" int sp_mlp_set_training_kernel(sp_mlp* m, int kind) {
    if (!m || (kind != SP_MLP_KERNEL_AUTO && kind != SP_MLP_KERNEL_TCGEN05 && kind != SP_MLP_KERNEL_MMA_SYNC))
        return SP_ERR_INVALID_ARGUMENT;
    if (kind == SP_MLP_KERNEL_TCGEN05 && m->H % 16 != 0)
        return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "tcgen05 training needs a hidden width that is a multiple of 16");
    std::lock_guard<std::mutex> g(m->ctx->mu);
    m->train_kind = kind;
    return SP_OK;
}

extern "C" int sp_mlp_fault(sp_mlp* m, int* fault) {
    if (!m || !fault) return SP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    int a = 0, b = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&a, m->step + 16, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && m->tc_err) e = cudaMemcpy(&b, m->tc_err, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return SP_ERR_TRANSFER;
    *fault = (a ? 1 : 0) | (b ? 2 : 0);
    return SP_OK;
}

extern "C" int sp_mlp_warm_start_device(sp_mlp* m, const double* d_params_soa, uint64_t stride, uint64_t rows,
                                        double* d_x0, void* stream) {
    if (!m || !d_params_soa || !d_x0) return SP_ERR_INVALID_ARGUMENT;
    if (rows == 0) return SP_OK;
    if (rows > kMaxRows || stride < rows) return mlp_fail(m->ctx, SP_ERR_INVALID_DIMENSION, "bad row count or stride");
    if (!m->io_set) return mlp_fail(m->ctx, SP_ERR_INVALID_ARGUMENT, "sp_mlp_set_io not called");
    std::lock_guard<std::mutex> g(m->ctx->mu);
    cudaSetDevice(m->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    ScratchOrder order(m->ctx, st);  // orders workspace reuse and growth after earlier users
    ProfScope prof(m->ctx, "mlp_warm_start", st);
    if (sp::mlp_warm_start(m, d_params_soa, (size_t)stride, (int)rows, d_x0, st) != cudaSuccess)
        return mlp_fail(m->ctx, SP_ERR_BACKEND, "warm-start inference launch");
    return SP_OK;
}

// Warm start for the learned sweep: parameters (SoA) -> network -> x0 (FP64).
namespace sp {
bool tc_eligible(const sp_mlp* m) { return mlptc::supported(m->d.n_in, m->d.n_out, m->H, m->L); }

cudaError_t tc_warm_start(sp_mlp* m, const double* params_soa, size_t stride, int rows, double* x0, cudaStream_t st) {
    mlptc::Args a{};
    const int img = mlptc::plan(m->d.n_in, m->d.n_out, m->H, m->L, &a);
    if (!m->tc_img) {
        cudaError_t e = cudaMalloc(&m->tc_img, img);
        if (e == cudaSuccess) e = cudaMalloc(&m->tc_bias, 4 * (size_t)a.bias_total);
        if (e == cudaSuccess) e = cudaMalloc(&m->tc_err, 4);
        if (e == cudaSuccess) e = cudaMemset(m->tc_err, 0, 4);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->ctx->device);
        if (e != cudaSuccess) return e;
    }
    // weights packed by an earlier call are complete before this call's kernels
    // start; weights packed now are not (the copies below precede the kernel)
    a.early_prologue = m->tc_dirty ? 0 : 1;
    if (m->tc_dirty) {
        cudaError_t e = mlptc::pack(m->params, m->woff.data(), a, m->tc_img, st);
        for (int l = 0; l < m->L && e == cudaSuccess; ++l)
            e = cudaMemcpyAsync(m->tc_bias + a.layer[l].bias_off, m->params + m->boff[l], 4 * (size_t)a.layer[l].N,
                                cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
        m->tc_dirty = false;
    }
    a.params_soa = params_soa;
    a.stride = stride;
    a.rows = rows;
    a.slots = m->io_slots;
    a.io = m->io;
    a.lin = m->has_lin ? m->lin_f32 : nullptr;
    a.bias = m->tc_bias;
    a.img = m->tc_img;
    a.x0 = x0;
    a.err = m->tc_err;
    a.teams_pref = tune_get(m->ctx, "mlp.teams", m->H, 0);  // tiles in flight per CTA (tuned)
    return mlptc::launch(a, m->num_sms, st);
}

// The linear warm start alone (SP_MLP_KERNEL_LINEAR) for a standalone call;
// the learned sweep evaluates the same formula in its draw kernel.
__global__ void linear_warm_kernel(const double* __restrict__ params_soa, size_t stride, int rows,
                                   const int* __restrict__ slots, const float* __restrict__ io,
                                   const float* __restrict__ lin, int n_in, int n_out, double* __restrict__ x0) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= rows) return;
    for (int k = 0; k < n_out; ++k) {
        float x = io[2 * n_in + k];
        for (int j = 0; j < n_in; ++j)
            x = fmaf(lin[k * n_in + j], __double2float_rn(params_soa[(size_t)slots[j] * stride + s]) - io[j], x);
        x0[(size_t)s * n_out + k] = (double)x;
    }
}

cudaError_t mlp_warm_start(sp_mlp* m, const double* params_soa, size_t stride, int rows, double* x0,
                           cudaStream_t st) {
    const int kind = m->kernel_kind;
    if (kind == SP_MLP_KERNEL_LINEAR) {
        linear_warm_kernel<<<(rows + 127) / 128, 128, 0, st>>>(params_soa, stride, rows, m->io_slots, m->io,
                                                               m->lin_f32, m->d.n_in, m->d.n_out, x0);
        return cudaGetLastError();
    }
    if (kind == SP_MLP_KERNEL_TCGEN05 || (kind == SP_MLP_KERNEL_AUTO && tc_eligible(m)))
        return tc_warm_start(m, params_soa, stride, rows, x0, st);
    if (kind != SP_MLP_KERNEL_LAYERED && m->H <= FH && m->L <= 9) {
        // fused path: activations never leave shared memory
        const size_t smem = (size_t)2 * FT * APITCH * 2 + (size_t)2 * FH * WPITCH * 2 + (size_t)FT * m->d.n_in * 4;
        if (!m->fused_ready) {
            cudaError_t e = cudaFuncSetAttribute(mlp_infer_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)((size_t)2 * FT * APITCH * 2 + (size_t)2 * FH * WPITCH * 2 +
                                                       (size_t)FT * 64 * 4));
            if (e != cudaSuccess) return e;
            m->fused_ready = true;
        }
        FusedArgs a{};
        a.params_soa = params_soa;
        a.stride = stride;
        a.rows = rows;
        a.slots = m->io_slots;
        a.io = m->io;
        a.lin = m->has_lin ? m->lin_f32 : nullptr;
        a.n_in = m->d.n_in;
        a.n_out = m->d.n_out;
        a.kin = m->kin;
        a.kout = m->kout;
        a.H = m->H;
        a.L = m->L;
        a.wt = m->wt_bf;
        a.params = m->params;
        for (int l = 0; l < m->L; ++l) {
            a.woff[l] = (int)m->woff[l];
            a.boff[l] = (int)m->boff[l];
        }
        a.x0 = x0;
        mlp_infer_fused<<<(rows + FT - 1) / FT, 256, smem, st>>>(a);
        return cudaGetLastError();
    }
    if (ensure_ws(m, rows) != SP_OK) return cudaErrorMemoryAllocation;
    const int rp = (rows + 63) & ~63;
    const float* io = m->io;
    pack_params<<<(rp * m->kin + 255) / 256, 256, 0, st>>>(params_soa, stride, rows, rp, m->io_slots, io,
                                                           io + m->d.n_in, m->d.n_in, m->kin, m->X);
    cudaError_t e = forward(m, rp, false, st);
    if (e != cudaSuccess) return e;
    unpack_outputs<<<(rows * m->d.n_out + 255) / 256, 256, 0, st>>>(
        m->Y, rows, m->kout, m->d.n_out, io + 2 * m->d.n_in, io + 2 * m->d.n_in + m->d.n_out, x0,
        m->has_lin ? m->lin : nullptr, params_soa, stride, m->io_slots, io, m->d.n_in);
    return cudaGetLastError();
}
int mlp_outputs(const sp_mlp* m) { return m->d.n_out; }
bool mlp_linear_only(const sp_mlp* m, DrawLaunch* d) {
    if (m->kernel_kind != SP_MLP_KERNEL_LINEAR || !m->has_lin) return false;
    d->lin = m->lin_f32;
    d->lin_io = m->io;
    d->lin_slots = m->io_slots;
    d->lin_nin = m->d.n_in;
    d->lin_nout = m->d.n_out;
    return true;
}
int mlp_max_slot(const sp_mlp* m) { return m->max_slot; }
bool mlp_linear_host(const sp_mlp* m, const float** lin, const float** io, const int** slots) {
    if (!m->has_lin || (int)m->h_lin.size() != m->d.n_out * m->d.n_in || (int)m->h_slots.size() != m->d.n_in ||
        (int)m->h_io.size() < 2 * m->d.n_in + m->d.n_out)
        return false;
    *lin = m->h_lin.data();
    *io = m->h_io.data();
    *slots = m->h_slots.data();
    return true;
}
bool mlp_inputs_drawn(const sp_mlp* m, const sp_param* params, int num_params) {
    for (int k : m->h_slots)
        if (k >= num_params || params[k].kind == SP_DRAW_FIXED) return false;
    return true;
}
uint64_t mlp_max_rows() { return kMaxRows; }
bool mlp_io_ready(const sp_mlp* m) { return m->io_set; }
sp_ctx* mlp_ctx(const sp_mlp* m) { return m->ctx; }
}  // namespace sp
