// Warm-start inference on the 5th-generation tensor cores (tcgen05, TMEM).
//
// One persistent CTA per SM keeps the whole network in shared memory: every
// layer's weight matrix W[N][K] is packed once, on the device, as FP16 into the
// tensor cores' K-major 128-byte-swizzled layout (8-row x 128-byte atoms,
// 16-byte chunks XOR-ed with the row), so a CTA fills its shared memory with
// one linear copy.  Up to four teams of 128 threads (four warps, warp q
// reading TMEM lanes 32q..32q+31) each own a 128-sample tile, an activation
// buffer in the same layout and 128 TMEM columns; thread t of a team owns
// sample row t of its tile from input to output:
//
//   stage inputs  centred parameters p - in_mean in FP32 (kept in registers
//                 for the FP32 linear term; relative error ~2^-24 /
//                 |p/in_mean - 1|), scaled to FP16 and written as row t of
//                 the A operand;
//   per layer     one thread issues K/16 tcgen05.mma (M=128, N=layer width,
//                 K=16, FP16 x FP16 -> FP32 in TMEM) and commits them to the
//                 team's mbarrier; after the wait every thread reads its
//                 TMEM lane 32 columns at a time (tcgen05.ld 32x32b.x32),
//                 adds the bias (FP32), applies GELU in packed FP16
//                 arithmetic (two activations per instruction) and writes
//                 the FP16 activations back as the next layer's A;
//   output        x0[k] = out_mean[k] + out_scale[k] y[k]
//                         + sum_j lin[k][j] (p_j - in_mean[j])    (FP32, then FP64)
//
// FP16 rather than the trainer's BF16: the inputs are normalised and the
// activations of a warm-start network stay far inside FP16's range, FP16
// keeps three more mantissa bits, and packed FP16 arithmetic halves the
// epilogue's instructions, which (not the tensor cores) bound a layer.
//
// With four teams a 65,536-sample sweep is one tile per team on 128 SMs: the
// teams' MMAs, TMEM reads and epilogues interleave on the SM, and no team
// waits for a second tile.  Every mbarrier wait is bounded: on a timeout the
// team fills its remaining samples' x0 with NaN (the Newton path then
// restarts those samples cold), raises the error flag, and the CTA frees
// its TMEM before it returns.
//
// Hidden width 256 (stream_kernel): the weights (304 KB for 10 -> 3x256 ->
// 12) no longer fit in shared memory, so they stream from L2 through a ring
// of 16 KB slots, each one K-block (64 K) of 128 weight rows (or the whole
// K-block of the 32-row output layer).  Roles per CTA (576 threads):
//   producer warp  one thread walks the CTA's fixed unit sequence and copies
//                  each unit into the next free slot with the TMA unit
//                  (full[slot] completes on the bytes, empty[slot] on the
//                  MMAs that read it);
//   MMA warp       one thread issues, for each (tile, layer) job in the
//                  same order, one tcgen05.mma (M = 128, N = unit rows,
//                  K = 16) per 16 K of every unit, commits each unit to its
//                  empty barrier and the job to the team's accumulator
//                  barrier;
//   two teams      of eight warps (warp w reads TMEM lanes 32 (w % 4) ..
//                  and column half (w / 4) % 2) each own a 128-sample tile,
//                  a 64 KB activation buffer and 256 TMEM columns, and run
//                  the epilogue of one layer while the tensor cores run the
//                  other team's layer: jobs alternate team 0 / team 1 layer
//                  by layer, so the MMA chain of one tile overlaps the
//                  bias + GELU + FP16 repack of the other.
// The weights never depend on the activations, so the producer runs ahead of
// the MMA warp by the ring's depth across layers and tiles.
//
// Scope: n_in <= 32, n_out <= 32, hidden width 64, 128 or 256, 1..4 hidden
// layers; the mma.sync kernel in mlp.cu serves every other shape.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <mutex>

#include "mlp_act.cuh"
#include "mlp_tc.h"
#include "pdl.cuh"

namespace sp {
namespace mlptc {

namespace {

constexpr int kTile = 128;      // samples per tile = MMA M
constexpr int kTeam = 128;      // threads per tile: 4 warps, one per TMEM lane quarter
constexpr int kMaxTeams = 4;    // tiles in flight per CTA (512 TMEM columns)
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 bytes apart (stride byte offset); the leading byte offset is unused
// for this layout; bits 46-47 hold the descriptor version (1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
}
// The same with FP16 A and B (the inference kernels).
__host__ __device__ constexpr uint32_t idesc_f16(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16_ss(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// Bulk copy global -> shared through the TMA unit (both addresses 16-byte
// aligned, bytes a multiple of 16), completing on mbar's transaction count.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(mbar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

// Named barrier of one team (128 threads) that also ANDs a predicate across it.
__device__ __forceinline__ bool team_all(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.b32 q, %1, 0;\n\t"
        "bar.red.and.pred p, %2, 128, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void team_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// FP64 <-> FP32 conversions on the integer pipe (GB300's FP64 pipe issues
// conversions slowly, and the kernel converts every input and output).
// Normal numbers only; zeros, subnormals, Inf and NaN take the ordinary path.
__device__ __forceinline__ float f64_to_f32(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 255) return __double2float_rn(x);
    const uint64_t m = b & ((1ULL << 52) - 1);
    uint32_t f = ((uint32_t)(b >> 32) & 0x80000000u) | ((uint32_t)e << 23) | (uint32_t)(m >> 29);
    const uint64_t rem = m & ((1ULL << 29) - 1), half = 1ULL << 28;
    f += (rem > half || (rem == half && (f & 1))) ? 1u : 0u;  // a carry rounds into the exponent
    return __uint_as_float(f);
}

__device__ __forceinline__ double f32_to_f64(float x) {
    const uint32_t f = __float_as_uint(x);
    const uint32_t e = (f >> 23) & 0xff;
    if (e == 0 || e == 255) return (double)x;
    const uint64_t b = ((uint64_t)(f & 0x80000000u) << 32) | ((uint64_t)(e - 127 + 1023) << 52) |
                       ((uint64_t)(f & 0x7fffffu) << 29);
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ uint32_t pack2h(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// GELU (tanh form) of two FP16 values in packed FP16 arithmetic: z/2 (1 +
// tanh(c z (1 + a z^2))), six instructions for two activations.  Large |z|
// saturates through infinities to z or 0 (tanh of +-inf is +-1), as the FP32
// form does.
__device__ __forceinline__ uint32_t gelu_h2(float z0, float z1) {
    const __half2 z = __floats2half2_rn(z0, z1);
    const __half2 ca = __float2half2_rn(act::kC * act::kA), c = __float2half2_rn(act::kC), hf = __float2half2_rn(0.5f);
    const __half2 u = __hmul2(z, z);
    const __half2 w = __hfma2(ca, u, c);
    const __half2 arg = __hmul2(z, w);
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<const uint32_t*>(&arg)));
    const __half2 hz = __hmul2(z, hf);
    const __half2 g = __hfma2(hz, *reinterpret_cast<const __half2*>(&t), hz);
    return *reinterpret_cast<const uint32_t*>(&g);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Byte offset of 16-byte chunk c (8 BF16 along K) of row r in a K-major,
// 128-byte-swizzled operand with `rows` rows: K-blocks of 64 elements are
// rows*128 bytes apart, 8-row atoms 1024 bytes apart.
__host__ __device__ __forceinline__ uint32_t sw128_offset(int rows, int r, int c) {
    return (uint32_t)((c >> 3) * rows * 128 + (r >> 3) * 1024 + (r & 7) * 128 + (((c & 7) ^ (r & 7)) << 4));
}

__global__ void pack_kernel(const float* __restrict__ wt, int N, int K, int Kp, unsigned char* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // one 16-byte chunk
    const int chunks = Kp / 8;
    if (i >= N * chunks) return;
    const int r = i / chunks, c = i % chunks;
    uint32_t w[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const int k0 = c * 8 + 2 * h;
        const float a = k0 < K ? wt[(size_t)r * K + k0] : 0.f;
        const float b = k0 + 1 < K ? wt[(size_t)r * K + k0 + 1] : 0.f;
        w[h] = pack2h(a, b);
    }
    *reinterpret_cast<uint4*>(dst + sw128_offset(N, r, c)) = make_uint4(w[0], w[1], w[2], w[3]);
}

// Shared-memory carve-up (byte offsets from the 1024-aligned base).
struct Carve {
    uint32_t abuf, bias, lin, io, slots, mbar, tslot, total;
};

__host__ __device__ inline Carve carve(const Args& a, int teams) {
    Carve c;
    c.abuf = (uint32_t)a.img_bytes;                       // multiple of 1024
    c.bias = c.abuf + (uint32_t)teams * kAbytes;
    c.lin = c.bias + 4u * (uint32_t)a.bias_total;
    c.io = c.lin + 4u * (uint32_t)(a.n_out * a.n_in);
    c.slots = c.io + 4u * (uint32_t)(2 * (a.n_in + a.n_out));
    c.mbar = (c.slots + 4u * (uint32_t)a.n_in + 7u) & ~7u;  // [kMaxTeams] teams, [kMaxTeams] weights
    c.tslot = c.mbar + 8u * (kMaxTeams + 1);
    c.total = c.tslot + 16u;
    return c;
}

constexpr uint32_t kSmemLimit = 227u * 1024u;

__host__ __device__ inline int teams_for(const Args& a) {
    for (int t = kMaxTeams; t >= 1; --t)
        if (1024u + carve(a, t).total <= kSmemLimit) return t;
    return 0;
}

__global__ void __launch_bounds__(kMaxTeams * kTeam, 1) infer_kernel(Args a, int teams) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // Under programmatic dependent launch a CTA can start while the previous
    // kernel (the parameter draws) drains.  Only the drawn parameters depend
    // on it: with early_prologue the weight copy, the constants and the TMEM
    // allocation run first, overlapping that kernel's tail.
    if (!a.early_prologue) pdl_wait();
    pdl_trigger();
    // 1024-byte alignment of the swizzled operands (the dynamic window may start lower)
    unsigned char* sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    const Carve cv = carve(a, teams);
    unsigned char* wimg = sm;
    float* bias_s = reinterpret_cast<float*>(sm + cv.bias);
    float* lin_s = reinterpret_cast<float*>(sm + cv.lin);
    float* io_s = reinterpret_cast<float*>(sm + cv.io);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + cv.mbar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + cv.tslot);

    int* slots_s = reinterpret_cast<int*>(sm + cv.slots);
    const uint32_t wbar = smem_u32(&mbar[kMaxTeams]);

    // team = tile slot; warp q of a team reads TMEM lanes 32q..32q+31 (its sample rows)
    const int tid = threadIdx.x, nthreads = teams * kTeam, team = tid / kTeam, tt = tid % kTeam, warp = tid >> 5;
    const int quarter = tt >> 5, row = tt;
    if (tid == 0) {
        for (int t = 0; t <= kMaxTeams; ++t)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[t])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the weight image (a.img_bytes, a multiple of 1024) by the TMA unit, 32 KB per copy
        mbar_expect_tx(wbar, (uint32_t)a.img_bytes);
        for (int off = 0; off < a.img_bytes; off += 32768) {
            const int len = a.img_bytes - off < 32768 ? a.img_bytes - off : 32768;
            bulk_g2s(smem_u32(wimg + off), static_cast<const unsigned char*>(a.img) + off, (uint32_t)len, wbar);
        }
    }
    for (int i = tid; i < a.bias_total; i += nthreads) bias_s[i] = a.bias[i];
    for (int i = tid; i < a.n_out * a.n_in; i += nthreads) lin_s[i] = a.lin ? a.lin[i] : 0.f;
    // in_mean, 1 / in_scale, out_mean, out_scale
    for (int i = tid; i < 2 * (a.n_in + a.n_out); i += nthreads)
        io_s[i] = (i >= a.n_in && i < 2 * a.n_in) ? 1.0f / a.io[i] : a.io[i];
    for (int i = tid; i < a.n_in; i += nthreads) slots_s[i] = a.slots[i];
    const uint32_t tcols = teams > 2 ? 512u : (teams > 1 ? 256u : 128u);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tcols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (a.early_prologue) pdl_wait();  // the drawn parameters are complete and visible
    const uint32_t tmem = *tmem_slot + (uint32_t)(team * 128);  // this team's 128 columns
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    unsigned char* abuf = sm + cv.abuf + team * kAbytes;
    const uint32_t abuf_s = smem_u32(abuf), wimg_s = smem_u32(wimg), mb = smem_u32(&mbar[team]);
    const int bar_id = 1 + team;
    const float* in_mean = io_s;
    const float* in_rscale = io_s + a.n_in;
    const float* out_mean = io_s + 2 * a.n_in;
    const float* out_scale = out_mean + a.n_out;

    const int ntiles = (a.rows + kTile - 1) / kTile;
    uint32_t phase = 0;
    bool ok = true, weights = false;
    int tile = blockIdx.x * teams + team;
    for (; tile < ntiles; tile += gridDim.x * teams) {
        const int s = tile * kTile + row;
        const bool live = s < a.rows;
        // inputs 0..31 of row `row` (chunks 0..3, kept in registers for the
        // linear term); chunks 4..7 of the first K-block are zero.  Every load
        // is issued before the first conversion (the conversion branches, so
        // interleaving them would serialise the loads' latencies)
        float pc[kMaxIn];
        {
            double raw[kMaxIn];
#pragma unroll
            for (int j = 0; j < kMaxIn; ++j)
                raw[j] = (j < a.n_in && live) ? __ldg(a.params_soa + (size_t)slots_s[j] * a.stride + s) : 0.0;
#pragma unroll
            for (int j = 0; j < kMaxIn; ++j) pc[j] = j < a.n_in && live ? f64_to_f32(raw[j]) - in_mean[j] : 0.f;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint32_t w[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int j = c * 8 + 2 * h;
                const float x0v = j < a.n_in ? pc[j] * in_rscale[j] : 0.f;
                const float x1v = j + 1 < a.n_in ? pc[j + 1] * in_rscale[j + 1] : 0.f;
                w[h] = pack2h(x0v, x1v);
            }
            *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
#pragma unroll
        for (int c = 4; c < 8; ++c)
            *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c)) = make_uint4(0u, 0u, 0u, 0u);
        for (int l = 0; l < a.L; ++l) {
            const Layer& ly = a.layer[l];
            fence_async_smem();  // generic-proxy writes of A -> visible to the tensor cores
            tc_before();
            team_sync(bar_id);
            tc_after();
            if (!weights) {  // the TMA copy of the weights (issued at the start) has landed
                ok = team_all(bar_id, mbar_wait(wbar, 0));
                weights = true;
                if (!ok) break;
            }
            if (tt == 0) {
                const uint32_t id = idesc_f16(ly.N);
                const uint32_t wb = wimg_s + (uint32_t)ly.img_off;
                for (int kb = 0; kb < ly.Kp / 64; ++kb)
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        mma_bf16_ss(tmem, sdesc(abuf_s + kb * kTile * 128 + k * 32),
                                    sdesc(wb + kb * ly.N * 128 + k * 32), id, (kb | k) != 0);
                mma_commit(mb);
            }
            ok = team_all(bar_id, mbar_wait(mb, phase));
            phase ^= 1;
            if (!ok) break;
            tc_after();
            const float* bias = bias_s + ly.bias_off;
            if (l + 1 < a.L) {
                for (int c0 = 0; c0 < ly.N; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
                    uint32_t w[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        w[i] = gelu_h2(v[2 * i] + bias[c0 + 2 * i], v[2 * i + 1] + bias[c0 + 2 * i + 1]);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c0 / 8 + q)) =
                            make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
                }
            } else {
                float v[32];
                tmem_ld32(tmem + lane_base, v);  // the output layer is 32 wide (n_out <= 32)
                if (live) {
#pragma unroll
                    for (int k = 0; k < 32; ++k) {
                        if (k < a.n_out) {
                            float x = out_mean[k] + out_scale[k] * (v[k] + bias[k]);
#pragma unroll
                            for (int j = 0; j < kMaxIn; ++j)
                                if (j < a.n_in) x = fmaf(lin_s[k * a.n_in + j], pc[j], x);
                            a.x0[(size_t)s * a.n_out + k] = f32_to_f64(x);
                        }
                    }
                }
            }
            tc_before();
        }
        if (!ok) break;
    }
    if (!ok) {
        // timeout: this team's remaining samples start cold (NaN warm start)
        if (tt == 0) atomicExch(a.err, 1);
        for (; tile < ntiles; tile += gridDim.x * teams) {
            const int s = tile * kTile + row;
            if (s < a.rows)
                for (int k = 0; k < a.n_out; ++k)
                    a.x0[(size_t)s * a.n_out + k] = __longlong_as_double(0x7ff8000000000000LL);
        }
    }
    // every MMA this CTA issued has completed (each team waited on its
    // commits, or gave up only after the bounded wait)
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tmem_slot), "r"(tcols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Hidden width 256: weights streamed from L2 (see the file comment).
constexpr int kSTeams = 2;                            // tiles in flight per CTA
constexpr int kSTeamWarps = 8;                        // warps per team
constexpr int kSTeamThreads = kSTeamWarps * 32;       // 256
constexpr int kSProducerWarp = kSTeams * kSTeamWarps;  // warp 16
constexpr int kSIssuerWarp = kSProducerWarp + 1;       // warp 17
constexpr int kSThreads = (kSIssuerWarp + 1) * 32;     // 576
constexpr uint32_t kSUnit = 16384;                    // one ring slot: 128 rows x 64 K of FP16
constexpr uint32_t kSAbytes = 128u * 256u * 2u;       // one activation tile: 128 samples x 256 FP16
constexpr int kSMaxSlots = 6;

struct SCarve {
    uint32_t abuf, ring, bias, lin, io, slots, mbar, flag, tslot, total;
};

__host__ __device__ inline SCarve scarve(const Args& a, int nslots) {
    SCarve c;
    c.abuf = 0;  // kSTeams x kSAbytes, 1024-aligned
    c.ring = kSTeams * kSAbytes;
    c.bias = c.ring + (uint32_t)nslots * kSUnit;
    c.lin = c.bias + 4u * (uint32_t)a.bias_total;
    c.io = c.lin + 4u * (uint32_t)(a.n_out * a.n_in);
    c.slots = c.io + 4u * (uint32_t)(2 * (a.n_in + a.n_out));
    c.mbar = (c.slots + 4u * (uint32_t)a.n_in + 7u) & ~7u;  // full[6], empty[6], ready[2], acc[2]
    c.flag = c.mbar + 8u * (2 * kSMaxSlots + 2 * kSTeams);
    c.tslot = c.flag + 16u;
    c.total = c.tslot + 16u;
    return c;
}

__host__ __device__ inline int stream_slots(const Args& a) {
    for (int s = kSMaxSlots; s >= 2; --s)
        if (1024u + scarve(a, s).total <= kSmemLimit) return s;
    return 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Bounded wait that also gives up when another role of the CTA has raised
// the abort flag (and raises it itself on a timeout).
__device__ __forceinline__ bool mbar_wait_ab(uint32_t mbar, uint32_t parity, volatile int* abort_flag) {
    const long long t0 = clock64();
    while (!mbar_try(mbar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void team_sync_n(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__device__ __forceinline__ bool team_all_n(int id, int n, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.b32 q, %1, 0;\n\t"
        "bar.red.and.pred p, %2, %3, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

// Units of layer ly: ceil(N / 128) row halves x Kp / 64 K-blocks, the row
// half outer; unit u covers rows nh*128 .. of K-block kb.
__device__ __forceinline__ int layer_units(const Layer& ly) { return ((ly.N + 127) / 128) * (ly.Kp / 64); }

__global__ void __launch_bounds__(kSThreads, 1) stream_kernel(Args a, int nslots) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // with early_prologue only the teams (which read the drawn parameters)
    // wait for the previous kernel: the set-up and the producer's first
    // weight copies overlap its tail (as in infer_kernel)
    if (!a.early_prologue) pdl_wait();
    pdl_trigger();
    unsigned char* sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    const SCarve cv = scarve(a, nslots);
    float* bias_s = reinterpret_cast<float*>(sm + cv.bias);
    float* lin_s = reinterpret_cast<float*>(sm + cv.lin);
    float* io_s = reinterpret_cast<float*>(sm + cv.io);
    int* slots_s = reinterpret_cast<int*>(sm + cv.slots);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + cv.mbar);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + cv.flag);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + cv.tslot);
    const uint32_t full0 = smem_u32(&mbar[0]), empty0 = smem_u32(&mbar[kSMaxSlots]);
    const uint32_t ready0 = smem_u32(&mbar[2 * kSMaxSlots]), acc0 = smem_u32(&mbar[2 * kSMaxSlots + kSTeams]);
    const uint32_t ring_s = smem_u32(sm + cv.ring);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int t = 0; t < 2 * kSMaxSlots + 2 * kSTeams; ++t)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[t])) : "memory");
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < a.bias_total; i += kSThreads) bias_s[i] = a.bias[i];
    for (int i = tid; i < a.n_out * a.n_in; i += kSThreads) lin_s[i] = a.lin ? a.lin[i] : 0.f;
    for (int i = tid; i < 2 * (a.n_in + a.n_out); i += kSThreads)
        io_s[i] = (i >= a.n_in && i < 2 * a.n_in) ? 1.0f / a.io[i] : a.io[i];
    for (int i = tid; i < a.n_in; i += kSThreads) slots_s[i] = a.slots[i];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (a.early_prologue && warp < kSProducerWarp) pdl_wait();  // teams: the drawn parameters are visible
    const uint32_t tmem = *tmem_slot;
    const int ntiles = (a.rows + kTile - 1) / kTile;
    // this CTA's tiles: k-th = blockIdx.x + k gridDim.x; tile k belongs to team k % 2
    const int my_tiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == kSProducerWarp) {
        if (lane == 0) {
            uint32_t g = 0;
            bool ok = true;
            for (int k2 = 0; ok && k2 < my_tiles; k2 += kSTeams)
                for (int l = 0; ok && l < a.L; ++l)
                    for (int T = 0; ok && T < kSTeams; ++T) {
                        if (k2 + T >= my_tiles) continue;
                        const Layer& ly = a.layer[l];
                        const int kbs = ly.Kp / 64, nu = layer_units(ly);
                        for (int u = 0; u < nu; ++u, ++g) {
                            const int nh = u / kbs, kb = u % kbs;
                            const uint32_t slot = g % (uint32_t)nslots;
                            if (!mbar_wait_ab(empty0 + 8 * slot, ((g / nslots) & 1u) ^ 1u, abort_flag)) {
                                ok = false;
                                break;
                            }
                            const int rows_u = min(128, ly.N - nh * 128);
                            const uint32_t bytes = (uint32_t)rows_u * 128u;
                            mbar_expect_tx(full0 + 8 * slot, bytes);
                            bulk_g2s(ring_s + slot * kSUnit,
                                     static_cast<const unsigned char*>(a.img) + ly.img_off + (size_t)kb * ly.N * 128 +
                                         (size_t)nh * 128 * 128,
                                     bytes, full0 + 8 * slot);
                        }
                    }
            if (!ok) {
                // copies still in flight land before the CTA releases its shared memory
                const uint32_t n_in_flight = g < (uint32_t)nslots ? g : (uint32_t)nslots;
                for (uint32_t j = g - n_in_flight; j < g; ++j) {
                    const long long t0 = clock64();
                    while (!mbar_try(full0 + 8 * (j % nslots), (j / nslots) & 1u))
                        if (clock64() - t0 > kWaitCycles) break;
                }
            }
        }
        __syncwarp();
    } else if (warp == kSIssuerWarp) {
        if (lane == 0) {
            uint32_t g = 0, jobs[kSTeams] = {0u, 0u};
            bool ok = true;
            for (int k2 = 0; ok && k2 < my_tiles; k2 += kSTeams)
                for (int l = 0; ok && l < a.L; ++l)
                    for (int T = 0; ok && T < kSTeams; ++T) {
                        if (k2 + T >= my_tiles) continue;
                        // team T's activations for layer l are in its buffer (and its
                        // previous accumulator has been read)
                        if (!mbar_wait_ab(ready0 + 8 * T, jobs[T] & 1u, abort_flag)) {
                            ok = false;
                            break;
                        }
                        tc_after();
                        const Layer& ly = a.layer[l];
                        const int kbs = ly.Kp / 64, nu = layer_units(ly);
                        const uint32_t abuf_s = smem_u32(sm + cv.abuf) + (uint32_t)T * kSAbytes;
                        for (int u = 0; u < nu; ++u, ++g) {
                            const int nh = u / kbs, kb = u % kbs;
                            const uint32_t slot = g % (uint32_t)nslots;
                            if (!mbar_wait_ab(full0 + 8 * slot, (g / nslots) & 1u, abort_flag)) {
                                ok = false;
                                break;
                            }
                            tc_after();
                            const int rows_u = min(128, ly.N - nh * 128);
                            const uint32_t id = idesc_f16(rows_u);
                            const uint32_t d = tmem + (uint32_t)(T * 256 + nh * 128);
                            const uint32_t ab = abuf_s + (uint32_t)kb * (kTile * 128), bb = ring_s + slot * kSUnit;
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                mma_bf16_ss(d, sdesc(ab + k * 32), sdesc(bb + k * 32), id, (kb | k) != 0);
                            mma_commit(empty0 + 8 * slot);  // the slot is free once these MMAs complete
                        }
                        if (!ok) break;
                        mma_commit(acc0 + 8 * T);  // the job's accumulator is complete
                        ++jobs[T];
                    }
        }
        __syncwarp();
    } else {
        // team T: warps 8T .. 8T+7; warp w reads TMEM lanes 32 (w % 4) .. and column half (w / 4) % 2
        const int T = warp / kSTeamWarps, wt = warp % kSTeamWarps, quarter = wt & 3, ch = wt >> 2;
        const int row = quarter * 32 + lane, bar_id = 1 + T;
        unsigned char* abuf = sm + cv.abuf + (uint32_t)T * kSAbytes;
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16, acc_b = acc0 + 8 * T;
        const float* in_mean = io_s;
        const float* in_rscale = io_s + a.n_in;
        const float* out_mean = io_s + 2 * a.n_in;
        const float* out_scale = out_mean + a.n_out;
        uint32_t jobs = 0;
        bool ok = true;
        int k = T;
        for (; k < my_tiles; k += kSTeams) {
            const int tile = (int)blockIdx.x + k * (int)gridDim.x;
            const int s = tile * kTile + row;
            const bool live = s < a.rows;
            if (ch == 0) {
                // inputs of row `row`: K-block 0, chunks 0..3 data, 4..7 zero
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    uint32_t w[4];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        const int j = c * 8 + 2 * h;
                        const float x0v = (j < a.n_in && live)
                                              ? (f64_to_f32(a.params_soa[(size_t)slots_s[j] * a.stride + s]) -
                                                 in_mean[j]) * in_rscale[j]
                                              : 0.f;
                        const float x1v = (j + 1 < a.n_in && live)
                                              ? (f64_to_f32(a.params_soa[(size_t)slots_s[j + 1] * a.stride + s]) -
                                                 in_mean[j + 1]) * in_rscale[j + 1]
                                              : 0.f;
                        w[h] = pack2h(x0v, x1v);
                    }
                    *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c)) = make_uint4(w[0], w[1], w[2], w[3]);
                }
#pragma unroll
                for (int c = 4; c < 8; ++c)
                    *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c)) = make_uint4(0u, 0u, 0u, 0u);
            }
            for (int l = 0; l < a.L; ++l) {
                // this layer's A operand is written (and the accumulator read): hand it to the MMA warp
                fence_async_smem();
                tc_before();
                team_sync_n(bar_id, kSTeamThreads);
                if (wt == 0 && lane == 0) mbar_arrive(ready0 + 8 * T);
                ok = team_all_n(bar_id, kSTeamThreads, mbar_wait_ab(acc_b, jobs & 1u, abort_flag));
                ++jobs;
                if (!ok) break;
                tc_after();
                const Layer& ly = a.layer[l];
                const float* bias = bias_s + ly.bias_off;
                if (l + 1 < a.L) {
                    const int half = ly.N / 2;  // columns per column half (128 for H = 256)
                    for (int c0 = ch * half; c0 < (ch + 1) * half; c0 += 32) {
                        float v[32];
                        tmem_ld32(tmem + lane_base + (uint32_t)(T * 256 + c0), v);
                        uint32_t w[16];
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            w[i] = gelu_h2(v[2 * i] + bias[c0 + 2 * i], v[2 * i + 1] + bias[c0 + 2 * i + 1]);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            *reinterpret_cast<uint4*>(abuf + sw128_offset(kTile, row, c0 / 8 + q)) =
                                make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
                    }
                } else if (ch == 0) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + (uint32_t)(T * 256), v);  // the output layer is 32 wide
                    if (live) {
                        // x[o] = out_mean + out_scale (y + b) + sum_j lin[o][j] (p_j - in_mean[j]);
                        // the centred inputs are read again, sixteen at a time with every load
                        // of a group issued before its first use
#pragma unroll
                        for (int o = 0; o < 32; ++o)
                            v[o] = o < a.n_out ? out_mean[o] + out_scale[o] * (v[o] + bias[o]) : 0.f;
                        const bool wide = a.n_out > 16;
                        for (int jb = 0; jb < a.n_in; jb += 16) {
                            float pc[16];
#pragma unroll
                            for (int t = 0; t < 16; ++t)
                                pc[t] = jb + t < a.n_in
                                            ? f64_to_f32(a.params_soa[(size_t)slots_s[jb + t] * a.stride + s]) - in_mean[jb + t]
                                            : 0.f;
#pragma unroll
                            for (int t = 0; t < 16; ++t) {
                                if (jb + t < a.n_in) {
                                    const int j = jb + t;
#pragma unroll
                                    for (int o = 0; o < 16; ++o)
                                        if (o < a.n_out) v[o] = fmaf(lin_s[o * a.n_in + j], pc[t], v[o]);
                                    if (wide) {
#pragma unroll
                                        for (int o = 16; o < 32; ++o)
                                            if (o < a.n_out) v[o] = fmaf(lin_s[o * a.n_in + j], pc[t], v[o]);
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int o = 0; o < 32; ++o)
                            if (o < a.n_out) a.x0[(size_t)s * a.n_out + o] = f32_to_f64(v[o]);
                    }
                }
            }
            if (!ok) break;
        }
        if (!ok) {
            // timeout: this team's remaining samples start cold (NaN warm start)
            if (wt == 0 && lane == 0) atomicExch(a.err, 1);
            if (ch == 0)
                for (; k < my_tiles; k += kSTeams) {
                    const int s = ((int)blockIdx.x + k * (int)gridDim.x) * kTile + row;
                    if (s < a.rows)
                        for (int o = 0; o < a.n_out; ++o)
                            a.x0[(size_t)s * a.n_out + o] = __longlong_as_double(0x7ff8000000000000LL);
                }
        }
    }
    // every MMA has completed (its team waited on the commit, or everything
    // gave up after a bounded wait) and no copy is in flight
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
}

// ---------------------------------------------------------------------------
// Training GEMMs: C[M][N] = A[M][K] B[N][K]^T with both operands K-major BF16
// (the layouts the trainer keeps, transposed copies included) and FP32
// accumulators in TMEM; the epilogues are those of the trainer's GEMMs.
// One CTA of four warps per 128 x BN output tile (BN <= 256) and K range
// (split-K along blockIdx.z): all threads copy 64-wide K-blocks of A and B
// into a two-stage ring of 128-byte-swizzled tiles (cp.async, zero-filled
// outside M, N and the K range); thread 0 issues the K-block's tcgen05.mma
// (M = 128, N = BN, K = 16 each) and commits them to the stage's mbarrier,
// which the copies into that stage wait for two K-blocks later; warp q then
// reads accumulator lanes 32q..32q+31 (its 32 output rows) for the epilogue.
// Waits are bounded: on a timeout the CTA raises *err, writes nothing and
// frees its TMEM after the copies and MMAs it started have drained.
constexpr int kGThreads = 128;
constexpr uint32_t kGAbytes = 128u * 128u;  // one K-block of A: 128 rows x 64 BF16

__host__ __device__ inline uint32_t gemm_stage_bytes(int bn) { return kGAbytes + (uint32_t)bn * 128u; }
__host__ __device__ inline uint32_t gemm_smem_bytes(int bn) { return 1024u + 2u * gemm_stage_bytes(bn) + 64u; }

__device__ __forceinline__ void cp_async16_zfill(uint32_t dst, const void* src, bool ok) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(ok ? 16 : 0) : "memory");
}

template <int EPI>
__global__ void __launch_bounds__(kGThreads) gemm_kernel(GemmTcArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    const int bn = g.bn;
    const uint32_t stage_bytes = gemm_stage_bytes(bn);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + 2 * stage_bytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + 2 * stage_bytes + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * bn;
    const int kb = blockIdx.z * g.k_split;
    const int ke = min(g.K, kb + g.k_split);
    const int natoms = ke > kb ? (ke - kb + 63) / 64 : 0;
    const uint32_t tcols = bn <= 32 ? 32u : (bn <= 64 ? 64u : (bn <= 128 ? 128u : 256u));
    if (tid == 0) {
        for (int t = 0; t < 2; ++t)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[t])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tcols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t base = smem_u32(sm);

    // K-block t into stage t & 1: A rows m0.., B rows n0.., 16-byte chunks
    auto load = [&](int t) {
        const uint32_t sa = base + (uint32_t)(t & 1) * stage_bytes, sb = sa + kGAbytes;
        const int k0 = kb + t * 64;
        for (int i = tid; i < (128 + bn) * 8; i += kGThreads) {
            const int r = i >> 3, c = i & 7, k = k0 + c * 8;
            if (r < 128) {
                const bool ok = m0 + r < g.M && k < ke;
                cp_async16_zfill(sa + sw128_offset(128, r, c), ok ? (const void*)(g.A + (size_t)(m0 + r) * g.lda + k)
                                                               : (const void*)g.A, ok);
            } else {
                const int rb = r - 128;
                const bool ok = n0 + rb < g.N && k < ke;
                cp_async16_zfill(sb + sw128_offset(bn, rb, c), ok ? (const void*)(g.B + (size_t)(n0 + rb) * g.ldb + k)
                                                                : (const void*)g.B, ok);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    bool ok = true;
    if (natoms > 0) load(0);
    for (int t = 0; t < natoms; ++t) {
        if (t + 1 < natoms) {
            // stage (t + 1) & 1 was last read by the MMAs of K-block t - 1
            // (the vote keeps the block's barriers uniform if a wait gives up)
            if (t >= 1) ok = __syncthreads_and(mbar_wait(smem_u32(&mbar[(t + 1) & 1]), (uint32_t)(((t - 1) >> 1) & 1)));
            if (!ok) break;
            load(t + 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        fence_async_smem();  // this thread's copies -> visible to the tensor cores
        tc_before();
        __syncthreads();
        tc_after();
        if (tid == 0) {
            const uint32_t sa = base + (uint32_t)(t & 1) * stage_bytes, sb = sa + kGAbytes;
            const int rem = ke - (kb + t * 64);
            const int ksteps = rem >= 64 ? 4 : (rem + 15) / 16;
            const uint32_t id = idesc_bf16(bn);
            for (int k = 0; k < ksteps; ++k)
                mma_bf16_ss(tmem, sdesc(sa + (uint32_t)k * 32u), sdesc(sb + (uint32_t)k * 32u), id, (t | k) != 0);
            mma_commit(smem_u32(&mbar[t & 1]));
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    // the last K-block's MMAs (every earlier commit completes before it)
    if (ok && natoms > 0) ok = mbar_wait(smem_u32(&mbar[(natoms - 1) & 1]), (uint32_t)(((natoms - 1) >> 1) & 1));
    ok = __syncthreads_and(ok);
    tc_after();
    if (!ok) {
        if (tid == 0) atomicExch(g.err, 1);
    } else {
        const int row = m0 + warp * 32 + lane;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        for (int c0 = 0; c0 < bn; c0 += 32) {
            float v[32];
            if (natoms > 0) {
                tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = 0.f;
            }
            if (row >= g.M) continue;
            // eight columns at a time: N and the tile width are multiples of 16, so a group
            // of eight is wholly inside or wholly outside the output; row-major outputs are
            // written 16 bytes per thread, the transposed copy 64 bytes per warp
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int col = n0 + c0 + 8 * q;
                if (c0 + 8 * q >= bn || col >= g.N) continue;
                const float* w = v + 8 * q;
                if (EPI == kEpiF32 || EPI == kEpiBiasF32) {
                    float o[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) o[j] = EPI == kEpiF32 ? w[j] : w[j] + g.bias[col + j];
                    float* dst = EPI == kEpiF32 ? g.C32 + ((size_t)blockIdx.z * g.M + row) * g.ldc + col
                                                : g.C32 + (size_t)row * g.ldc + col;
                    reinterpret_cast<float4*>(dst)[0] = make_float4(o[0], o[1], o[2], o[3]);
                    reinterpret_cast<float4*>(dst)[1] = make_float4(o[4], o[5], o[6], o[7]);
                } else {
                    uint32_t hz[4], hh[4];
                    __nv_bfloat16 hb[8];
#pragma unroll
                    for (int j = 0; j < 8; j += 2) {
                        float a0, a1;
                        if (EPI == kEpiBiasGelu) {
                            const float z0 = w[j] + g.bias[col + j], z1 = w[j + 1] + g.bias[col + j + 1];
                            hz[j / 2] = pack2(z0, z1);
                            a0 = act::gelu(z0);
                            a1 = act::gelu(z1);
                        } else {
                            const __nv_bfloat162 zin =
                                *reinterpret_cast<const __nv_bfloat162*>(g.Zin + (size_t)row * g.ld + col + j);
                            a0 = w[j] * act::gelu_grad(__low2float(zin));
                            a1 = w[j + 1] * act::gelu_grad(__high2float(zin));
                        }
                        hh[j / 2] = pack2(a0, a1);
                        hb[j] = __float2bfloat16(a0);
                        hb[j + 1] = __float2bfloat16(a1);
                    }
                    if (EPI == kEpiBiasGelu)
                        *reinterpret_cast<uint4*>(g.Z + (size_t)row * g.ld + col) = make_uint4(hz[0], hz[1], hz[2], hz[3]);
                    *reinterpret_cast<uint4*>(g.H + (size_t)row * g.ld + col) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
#pragma unroll
                    for (int j = 0; j < 8; ++j) g.Ht[(size_t)(col + j) * g.ldt + row] = hb[j];
                }
            }
        }
    }
    // every MMA has completed (waited above, or the bounded wait gave up)
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols) : "memory");
}

}  // namespace

bool supported(int n_in, int n_out, int hidden, int gemm_layers) {
    return n_in >= 1 && n_in <= kMaxIn && n_out >= 1 && n_out <= 32 &&
           (hidden == 64 || hidden == 128 || hidden == 256) && gemm_layers >= 2 && gemm_layers <= kMaxLayers;
}

int plan(int n_in, int n_out, int hidden, int gemm_layers, Args* a) {
    int off = 0, boff = 0;
    a->L = gemm_layers;
    for (int l = 0; l < gemm_layers; ++l) {
        Layer& ly = a->layer[l];
        ly.N = (l == gemm_layers - 1) ? 32 : hidden;  // padded output width (kout)
        ly.K = (l == 0) ? 32 : hidden;                // padded input width as stored (kin)
        ly.Kp = (ly.K + 63) & ~63;
        ly.img_off = off;
        ly.bias_off = boff;
        off += ly.N * ly.Kp * 2;
        boff += ly.N;
    }
    a->img_bytes = off;
    a->bias_total = boff;
    a->n_in = n_in;
    a->n_out = n_out;
    return off;
}

static bool streams(const Args& a) { return a.layer[0].N == 256; }

size_t smem_bytes(const Args& a) {
    if (streams(a)) {
        const int s = stream_slots(a);
        return s ? 1024 + (size_t)scarve(a, s).total : 0;
    }
    const int t = teams_for(a);
    return t ? 1024 + (size_t)carve(a, t).total : 0;
}

cudaError_t pack(const float* wt, const size_t* woff, const Args& a, void* img, cudaStream_t st) {
    for (int l = 0; l < a.L; ++l) {
        const Layer& ly = a.layer[l];
        const int n = ly.N * ly.Kp / 8;
        pack_kernel<<<(n + 255) / 256, 256, 0, st>>>(wt + woff[l], ly.N, ly.K, ly.Kp,
                                                     static_cast<unsigned char*>(img) + ly.img_off);
    }
    return cudaGetLastError();
}

// Raises the kernels' dynamic shared-memory limit once per device.
static cudaError_t configure_device() {
    static std::mutex mu;
    static bool configured[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 0 && dev < 64 && configured[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stream_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit);
    if (e == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = true;
    return e;
}

cudaError_t launch(const Args& a, int num_sms, cudaStream_t st) {
    cudaError_t e = configure_device();
    if (e != cudaSuccess) return e;
    const int ntiles = (a.rows + kTile - 1) / kTile;
    if (streams(a)) {
        const int nslots = stream_slots(a);
        if (nslots == 0) return cudaErrorInvalidValue;
        const size_t smem = 1024 + (size_t)scarve(a, nslots).total;
        // one CTA per SM; a CTA takes tiles blockIdx.x + k gridDim.x
        int grid = ntiles < num_sms ? ntiles : num_sms;
        if (grid < 1) return cudaSuccess;
        return launch_chained(stream_kernel, dim3(grid), dim3(kSThreads), smem, st, a, nslots);
    }
    int teams = teams_for(a);
    if (teams == 0) return cudaErrorInvalidValue;
    if (a.teams_pref > 0 && a.teams_pref < teams) teams = a.teams_pref;
    const size_t smem = 1024 + (size_t)carve(a, teams).total;
    int grid = (ntiles + teams - 1) / teams;
    if (grid > num_sms) grid = num_sms;
    if (grid < 1) return cudaSuccess;
    return launch_chained(infer_kernel, dim3(grid), dim3(teams * kTeam), smem, st, a, teams);
}

bool gemm_supported(const GemmTcArgs& g) {
    return g.M > 0 && g.N > 0 && g.N % 16 == 0 && g.K % 8 == 0 && g.k_split % 8 == 0 && g.k_split > 0 &&
           g.lda % 8 == 0 && g.ldb % 8 == 0 && g.epi >= kEpiF32 && g.epi <= kEpiGeluBwd && g.err != nullptr;
}

cudaError_t gemm(GemmTcArgs g, int splits, cudaStream_t st) {
    if (!gemm_supported(g) || splits < 1) return cudaErrorInvalidValue;
    static std::mutex mu;
    static bool configured[64] = {};
    static int sms_of[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (dev < 0 || dev >= 64 || !configured[dev]) {
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            const int lim = (int)gemm_smem_bytes(256);
            e = cudaFuncSetAttribute(gemm_kernel<kEpiF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(gemm_kernel<kEpiBiasF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(gemm_kernel<kEpiBiasGelu>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(gemm_kernel<kEpiGeluBwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
            if (e != cudaSuccess) return e;
            if (dev >= 0 && dev < 64) {
                configured[dev] = true;
                sms_of[dev] = sms;
            }
        } else {
            sms = sms_of[dev];
        }
    }
    // tile width: the widest (<= 256, a multiple of 16) that still gives every
    // SM a tile; these GEMMs are small, so CTAs in flight matter more than
    // the reuse of a wide tile
    const long long mt = (g.M + 127) / 128;
    int bn = g.N <= 256 ? g.N : 256;
    while (bn > 32 && mt * ((g.N + bn - 1) / bn) * splits < sms) bn = ((bn / 2 + 15) / 16) * 16;
    g.bn = bn;
    const uint32_t smem = gemm_smem_bytes(g.bn);
    const dim3 grid((unsigned)((g.M + 127) / 128), (unsigned)((g.N + g.bn - 1) / g.bn), (unsigned)splits);
    switch (g.epi) {
        case kEpiF32: gemm_kernel<kEpiF32><<<grid, kGThreads, smem, st>>>(g); break;
        case kEpiBiasF32: gemm_kernel<kEpiBiasF32><<<grid, kGThreads, smem, st>>>(g); break;
        case kEpiBiasGelu: gemm_kernel<kEpiBiasGelu><<<grid, kGThreads, smem, st>>>(g); break;
        default: gemm_kernel<kEpiGeluBwd><<<grid, kGThreads, smem, st>>>(g); break;
    }
    return cudaGetLastError();
}

}  // namespace mlptc
}  // namespace sp
