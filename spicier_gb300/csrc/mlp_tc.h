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
    Layer layer[kMaxLayers];
};

// Shapes these kernels run: n_in <= 32, n_out <= 32, 2..5 GEMM layers, and
// hidden width 64 or 128 (every weight resident in shared memory) or 256
// (weights streamed from L2 through a ring of shared-memory slots).
bool supported(int n_in, int n_out, int hidden, int gemm_layers);
// Fills the layer table of `a` (and n_in, n_out); returns the image size.
int plan(int n_in, int n_out, int hidden, int gemm_layers, Args* a);
size_t smem_bytes(const Args& a);
// Packs the row-major BF16 weights (layer l at wt + woff[l]) into the image.
cudaError_t pack(const __nv_bfloat16* wt, const size_t* woff, const Args& a, void* img, cudaStream_t st);
cudaError_t launch(const Args& a, int num_sms, cudaStream_t st);

}  // namespace mlptc
}  // namespace sp
