// Interface of the tcgen05 warm-start inference kernel (mlp_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sp {
namespace mlptc {

constexpr int kMaxIn = 32;      // network inputs (one 64-element K-block, padded)
constexpr int kMaxLayers = 5;   // GEMM layers (hidden layers + output)
constexpr int kAbytes = 128 * 128 * 2;  // one activation tile: 128 samples x 128 BF16

struct Layer {
    int N;        // output width (hidden, or 32 for the padded output layer)
    int K;        // input width as stored in the row-major weights
    int Kp;       // K rounded up to 64 (one swizzle atom per 64 elements)
    int img_off;  // byte offset of this layer in the packed weight image
    int bias_off; // offset of this layer's bias in the bias array
};

struct Args {
    const double* params_soa;  // [slot][stride]
    size_t stride;
    int rows;
    const int* slots;          // [n_in] parameter slots of the inputs
    const float* io;           // in_mean[n_in], in_scale[n_in], out_mean[n_out], out_scale[n_out]
    const float* lin;          // [n_out][n_in] FP32 linear term, or nullptr
    const float* bias;         // concatenated biases (bias_off per layer)
    const void* img;           // packed weight image (img_bytes)
    double* x0;                // [rows][n_out]
    int* err;                  // set to 1 when a bounded wait timed out
    int n_in, n_out, L, img_bytes, bias_total;
    int teams_pref;            // 0: the most tiles in flight that fit; else at most this many (tuned)
    int early_prologue;        // 1: the weights, biases and I/O constants were complete before the previous
                               // kernel of the stream began, so the CTA loads them before its dependency wait
    Layer layer[kMaxLayers];
};

// Shapes these kernels run: n_in <= 32, n_out <= 32, 2..5 GEMM layers, and
// hidden width 64 or 128 (every weight resident in shared memory) or 256
// (weights streamed from L2 through a ring of shared-memory slots).
bool supported(int n_in, int n_out, int hidden, int gemm_layers);
// Fills the layer table of `a` (and n_in, n_out); returns the image size.
int plan(int n_in, int n_out, int hidden, int gemm_layers, Args* a);
size_t smem_bytes(const Args& a);
// Packs the row-major FP32 weights (layer l at wt + woff[l]) into the image as FP16.
cudaError_t pack(const float* wt, const size_t* woff, const Args& a, void* img, cudaStream_t st);
cudaError_t launch(const Args& a, int num_sms, cudaStream_t st);

// Training GEMM C[M][N] = A[M][K] B[N][K]^T (BF16, K-major operands, FP32
// accumulation) with one of the trainer's epilogues:
//   kEpiF32       C32[z][M][ldc] = the partial sum of split z (split-K)
//   kEpiBiasF32   C32[M][ldc] = C + bias
//   kEpiBiasGelu  Z = C + bias, H = gelu(Z) (BF16 [M][ld]) and Ht = H^T ([N][ldt])
//   kEpiGeluBwd   H = Ht^T = C * gelu'(Zin) (BF16)
enum { kEpiF32 = 0, kEpiBiasF32 = 1, kEpiBiasGelu = 2, kEpiGeluBwd = 3 };
struct GemmTcArgs {
    const __nv_bfloat16* A;
    int lda;
    const __nv_bfloat16* B;
    int ldb;
    int M, N, K;
    int k_split;  // K elements per blockIdx.z (multiple of 8)
    float* C32;
    int ldc;
    const float* bias;
    __nv_bfloat16* Z;
    __nv_bfloat16* H;
    __nv_bfloat16* Ht;
    const __nv_bfloat16* Zin;
    int ld, ldt;
    int epi;
    int* err;  // set to 1 when a bounded wait timed out
    int bn;    // tile width (set by gemm())
};
// N a multiple of 16, K, k_split, lda and ldb multiples of 8.
bool gemm_supported(const GemmTcArgs& g);
cudaError_t gemm(GemmTcArgs g, int splits, cudaStream_t st);

}  // namespace mlptc
}  // namespace sp
