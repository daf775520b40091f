// Tensor-core (tcgen05) inference of the preconditioner network: the three
// layers of one 128-pair tile run back to back in one CTA.  BF16 operands sit
// in shared memory in the K-major core-matrix layout, both hidden layers
// accumulate in FP32 in tensor memory (256 columns: layer 1 in columns 0-127,
// layer 2 in 128-255), and the epilogues (bias, tanh, BF16 rounding, the
// 128 -> 2 output layer) run on the four warps that own the 128 TMEM lanes.
// One elected thread issues the MMAs; completion is signalled on an mbarrier
// through tcgen05.commit and every wait is bounded.
#include "common.cuh"
#include "kernels.cuh"
#include "precond.cuh"
#include "umma.cuh"

namespace bem {

namespace {
constexpr int TM = 128, NF_ = 16, NH_ = 128;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH_ * NF_, OFF_W2 = OFF_B1 + NH_, OFF_B2 = OFF_W2 + NH_ * NH_,
              OFF_W3 = OFF_B2 + NH_, OFF_B3 = OFF_W3 + 2 * NH_;
// shared memory map (bytes)
constexpr uint32_t S_X = 0, S_W1 = 4096, S_H1 = 8192, S_W2 = 40960, S_F = 73728;
constexpr uint32_t S_BAR = S_F + 4 * (NH_ + NH_ + 2 * NH_ + 2 + 2);  // 8-byte aligned
constexpr uint32_t S_TMEM = S_BAR + 8;
// requested dynamic shared memory: large enough that at most two CTAs share an
// SM, so their 2 x 256 tensor-memory columns always fit
constexpr uint32_t SMEM_BYTES = 110 * 1024;
constexpr uint32_t TMEM_COLS = 256;
}  // namespace

__device__ __forceinline__ float bf16round(float x) { return __bfloat162float(__float2bfloat16(x)); }
// The activation: the special-function unit's tanh (PTX tanh.approx.f32,
// absolute error about 2^-11), well inside the BF16 rounding (2^-9 relative)
// applied to every activation next.
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// Two floats as one BF16 pair (the first in the low half, at the lower address).
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
    const __nv_bfloat162 x = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&x);
}

__global__ void __launch_bounds__(TM) mlp_infer_tc_kernel(int64_t P, const float* __restrict__ F,
                                                          const float* __restrict__ w, float* __restrict__ O,
                                                          const int64_t* __restrict__ dst,
                                                          const float* __restrict__ scale, float2* __restrict__ M,
                                                          int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __nv_bfloat16* sW1 = reinterpret_cast<__nv_bfloat16*>(smem + S_W1);
    __nv_bfloat16* sW2 = reinterpret_cast<__nv_bfloat16*>(smem + S_W2);
    float* sb1 = reinterpret_cast<float*>(smem + S_F);
    float* sb2 = sb1 + NH_;
    float* sW3 = sb2 + NH_;
    float* sb3 = sW3 + 2 * NH_;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + S_BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + S_TMEM);
    const int tid = threadIdx.x, warp = tid >> 5;

    // weights, BF16-rounded, into the operand layouts (byte offsets / 2 = element index)
    for (int t = tid; t < NH_ * NF_; t += TM) {
        int n = t / NF_, k = t % NF_;
        sW1[umma_kmajor_offset(n, k, NF_) / 2] = __float2bfloat16(w[OFF_W1 + t]);
    }
    for (int t = tid; t < NH_ * NH_; t += TM) {
        int n = t / NH_, k = t % NH_;
        sW2[umma_kmajor_offset(n, k, NH_) / 2] = __float2bfloat16(w[OFF_W2 + t]);
    }
    for (int t = tid; t < NH_; t += TM) {
        sb1[t] = bf16round(w[OFF_B1 + t]);
        sb2[t] = bf16round(w[OFF_B2 + t]);
        sW3[t] = bf16round(w[OFF_W3 + t]);
        sW3[NH_ + t] = bf16round(w[OFF_W3 + NH_ + t]);
    }
    if (tid < 2) sb3[tid] = bf16round(w[OFF_B3 + tid]);
    if (warp == 0) tmem_alloc(tmem_slot, TMEM_COLS);
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = umma_idesc_bf16_f32(TM, NH_);
    const uint32_t base = smem_u32(smem);
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    uint32_t phase = 0;
    const int64_t ntiles = (P + TM - 1) / TM;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t p = tile * TM + tid;
        // layer-1 operand: this thread's feature row (64 bytes, four 16-byte
        // loads), eight BF16 features per 16-byte store of the core-matrix row
        {
            float4 f[NF_ / 4];
#pragma unroll
            for (int q = 0; q < NF_ / 4; ++q)
                f[q] = p < P ? reinterpret_cast<const float4*>(F + p * NF_)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < NF_ / 8; ++j)
                *reinterpret_cast<uint4*>(smem + S_X + umma_kmajor_offset(tid, 8 * j, NF_)) =
                    make_uint4(bf16x2_bits(f[2 * j].x, f[2 * j].y), bf16x2_bits(f[2 * j].z, f[2 * j].w),
                               bf16x2_bits(f[2 * j + 1].x, f[2 * j + 1].y), bf16x2_bits(f[2 * j + 1].z, f[2 * j + 1].w));
        }
        fence_proxy_async_shared();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            umma_bf16(tmem, umma_smem_desc(base + S_X, 128, 256), umma_smem_desc(base + S_W1, 128, 256), idesc, 0);
            umma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase)) != 0;
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        // epilogue 1: bias, tanh, BF16 -> layer-2 operand
        for (int c0 = 0; c0 < NH_; c0 += 32) {
            float v[32];
            tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint32_t h[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int i = 8 * j + 2 * e;
                    h[e] = bf16x2_bits(tanh_sfu(v[i] + sb1[c0 + i]), tanh_sfu(v[i + 1] + sb1[c0 + i + 1]));
                }
                *reinterpret_cast<uint4*>(smem + S_H1 + umma_kmajor_offset(tid, c0 + 8 * j, NH_)) =
                    make_uint4(h[0], h[1], h[2], h[3]);
            }
        }
        fence_proxy_async_shared();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            for (int kk = 0; kk < NH_ / 16; ++kk)
                umma_bf16(tmem + NH_, umma_smem_desc(base + S_H1 + 256 * kk, 128, 2048),
                          umma_smem_desc(base + S_W2 + 256 * kk, 128, 2048), idesc, kk > 0 ? 1u : 0u);
            umma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(bar, phase)) != 0;
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        // epilogue 2: bias, tanh, BF16, then the 128 -> 2 output layer in FP32
        float o0 = sb3[0], o1 = sb3[1];
        for (int c0 = 0; c0 < NH_; c0 += 32) {
            float v[32];
            tmem_ld32(tmem + lane_base + (uint32_t)(NH_ + c0), v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                float h = bf16round(tanh_sfu(v[i] + sb2[c0 + i]));
                o0 = fmaf(sW3[c0 + i], h, o0);
                o1 = fmaf(sW3[NH_ + c0 + i], h, o1);
            }
        }
        if (p < P) {
            if (O) {
                O[2 * p] = o0;
                O[2 * p + 1] = o1;
            }
            if (M) M[dst[p]] = make_float2(scale[p] * o0, scale[p] * o1);
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (!ok) {
        if (tid == 0) atomicOr(err, DEVERR_MBAR_TIMEOUT);
        mbar_wait_bounded(bar, phase);  // let an outstanding MMA drain before freeing its columns
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

void mlp_infer_tc(Context& c, const LearnedNet& net, int64_t P, const float* F, float* O, const int64_t* dst,
                  const float* scale, float2* M, bool check) {
    if (P <= 0) return;
    int* err = device_err(c);
    if (check) BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    // the same constant on every call: safe from any thread and on every
    // device (the attribute is per device)
    BEM_CUDA(cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    int sms = 0;
    BEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    const int64_t ntiles = (P + TM - 1) / TM;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, 2 * (int64_t)sms);
    mlp_infer_tc_kernel<<<grid, TM, SMEM_BYTES, c.stream>>>(P, F, net.w.as<float>(), O, dst, scale, M, err);
    BEM_CHECK_LAUNCH(&c);
    if (check) check_device_err(c);
}

}  // namespace bem
