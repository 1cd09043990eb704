// pg_filter.cu -- learned candidate-pair filter (sm_103a).
//
// PASTIS prunes candidate pairs before alignment by their k-mer overlap only:
// count <= ckthr or score <= mosthr drops a pair (src/DistPWRunner.cpp:48-54).
// This file adds a learned version of that prune: a 16 -> 64 -> 64 -> 1 ReLU
// network over k-mer overlap features of each pair, with BF16 weights and FP32
// accumulation on the tensor cores (mma.sync m16n8k16), trained by the
// hand-written forward / backward / Adam kernels below on pairs labelled by
// this library's own aligner.  pg_align_filtered aligns only the pairs the
// network keeps; the plain aligner stays the reference and judges its recall.
//
// Features of a pair (row sequence length m, column length n, L = max(m, n),
// k-mer count c, k-mer score s, seeds (r0, c0), (r1, c1)), fixed scaling:
//   0 log2(1+c)/4       1 s/32             2 [c >= 2]
//   3 (c0-r0)/L         4 (c1-r1)/L*[c>=2]  5 |(c0-r0)-(c1-r1)|/L*[c>=2]
//   6 r0/m              7 c0/n             8 best seed diagonal window (below)
//   9 log2(m)/12       10 log2(n)/12      11 |log2(m/n)|
//  12..15 |fraction difference| of the two sequences in four residue groups:
//         hydrophobic AVLIMFWC, polar NQSTYGP, positive RKH, negative DE
// Seed diagonal window: the mean substitution score over the 64 positions of
// a seed's diagonal from 32 before its start (positions outside either
// sequence skipped), divided by 4; the larger of the two seeds when the pair
// has two different ones.  It is the ungapped check BLAST-style seeders make
// before a gapped extension.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pastis_gb300.h"

int pg_internal_seqs(const pg_ctx *c, const uint8_t **rseq, const uint64_t **roffs, uint64_t *nr,
                     const uint8_t **cseq, const uint64_t **coffs, uint64_t *nc, int *device,
                     void **stream, int *mode);
int pg_internal_fail(int code, const char *msg);
int pg_internal_score(const pg_ctx *c, const int8_t **d_sm);

namespace {

constexpr int NF = PG_FILTER_FEATURES;   // 16
constexpr int NH = 64;
// parameter block (FP32 master copy); weights stored output-major
constexpr int P_W1 = 0;                  // [64][16]
constexpr int P_B1 = P_W1 + NH * NF;     // [64]
constexpr int P_W2 = P_B1 + NH;          // [64][64]
constexpr int P_B2 = P_W2 + NH * NH;     // [64]
constexpr int P_W3 = P_B2 + NH;          // [64]
constexpr int P_B3 = P_W3 + NH;          // [1]
constexpr int NPARAM = P_B3 + 1;

constexpr int FWARPS = 4;                // warps per block in the MLP kernels

#define FCU(call)                                                                  \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return pg_internal_fail(e_ == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, \
                                    cudaGetErrorString(e_));                       \
    } while (0)

// ------------------------------------------------------------ tensor cores
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t ld_u32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// weights as the MLP kernels read them from shared memory
struct SmemW {
    __nv_bfloat16 w1t[NH * NF];   // [out][in]      layer-1 B operand
    __nv_bfloat16 w2t[NH * NH];   // [out][in]      layer-2 B operand
    __nv_bfloat16 w2[NH * NH];    // [in][out]      backward B operand
    float b1[NH], b2[NH], w3[NH], b3;
};

__device__ void load_weights(SmemW &s, const float *P)
{
    for (int k = threadIdx.x; k < NH * NF; k += blockDim.x) s.w1t[k] = __float2bfloat16_rn(P[P_W1 + k]);
    for (int k = threadIdx.x; k < NH * NH; k += blockDim.x) {
        const int o = k / NH, i = k % NH;
        const __nv_bfloat16 v = __float2bfloat16_rn(P[P_W2 + k]);
        s.w2t[k] = v;
        s.w2[i * NH + o] = v;
    }
    for (int k = threadIdx.x; k < NH; k += blockDim.x) {
        s.b1[k] = P[P_B1 + k];
        s.b2[k] = P[P_B2 + k];
        s.w3[k] = P[P_W3 + k];
    }
    if (threadIdx.x == 0) s.b3 = P[P_B3];
}

// Forward pass of 16 samples starting at row `base` of X (bf16 [n][16]).
// Thread (g = lane/4, t = lane%4) ends up with the rows g and g+8 of h1 / h2 in
// the mma accumulator layout, and the logits of those two rows.
struct Tile {
    float h1[8][4];   // relu(x W1 + b1), fp32
    float h2[8][4];   // relu(h1_bf16 W2 + b2)
    float z0, z1;     // logits of rows g, g+8
};

__device__ __forceinline__ void forward_tile(const SmemW &s, const __nv_bfloat16 *X, uint64_t n,
                                             uint64_t base, Tile &T)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint64_t r0 = base + g, r1 = base + g + 8;
    uint32_t a[4];
    a[0] = r0 < n ? ld_u32(X + r0 * NF + 2 * t) : 0u;
    a[1] = r1 < n ? ld_u32(X + r1 * NF + 2 * t) : 0u;
    a[2] = r0 < n ? ld_u32(X + r0 * NF + 2 * t + 8) : 0u;
    a[3] = r1 < n ? ld_u32(X + r1 * NF + 2 * t + 8) : 0u;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16 *w = s.w1t + (nt * 8 + g) * NF + 2 * t;
        mma16816(d, a, ld_u32(w), ld_u32(w + 8));
        const int c = nt * 8 + 2 * t;
        T.h1[nt][0] = fmaxf(d[0] + s.b1[c], 0.f);
        T.h1[nt][1] = fmaxf(d[1] + s.b1[c + 1], 0.f);
        T.h1[nt][2] = fmaxf(d[2] + s.b1[c], 0.f);
        T.h1[nt][3] = fmaxf(d[3] + s.b1[c + 1], 0.f);
    }
    uint32_t a2[4][4];
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
        a2[kc][0] = pack_bf16(T.h1[2 * kc][0], T.h1[2 * kc][1]);
        a2[kc][1] = pack_bf16(T.h1[2 * kc][2], T.h1[2 * kc][3]);
        a2[kc][2] = pack_bf16(T.h1[2 * kc + 1][0], T.h1[2 * kc + 1][1]);
        a2[kc][3] = pack_bf16(T.h1[2 * kc + 1][2], T.h1[2 * kc + 1][3]);
    }
    float z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
            const __nv_bfloat16 *w = s.w2t + (nt * 8 + g) * NH + kc * 16 + 2 * t;
            mma16816(d, a2[kc], ld_u32(w), ld_u32(w + 8));
        }
        const int c = nt * 8 + 2 * t;
        T.h2[nt][0] = fmaxf(d[0] + s.b2[c], 0.f);
        T.h2[nt][1] = fmaxf(d[1] + s.b2[c + 1], 0.f);
        T.h2[nt][2] = fmaxf(d[2] + s.b2[c], 0.f);
        T.h2[nt][3] = fmaxf(d[3] + s.b2[c + 1], 0.f);
        z0 += T.h2[nt][0] * s.w3[c] + T.h2[nt][1] * s.w3[c + 1];
        z1 += T.h2[nt][2] * s.w3[c] + T.h2[nt][3] * s.w3[c + 1];
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    T.z0 = z0 + s.b3;
    T.z1 = z1 + s.b3;
}

// ----------------------------------------------------------------- kernels
__global__ void k_composition(const uint8_t *seq, const uint64_t *offs, uint64_t nseq, float4 *comp)
{
    // residue group of each code in ARNDCQEGHILKMFPSTWYVBZX*J; 4 = none
    const uint8_t grp[25] = {0, 2, 1, 3, 0, 1, 3, 1, 2, 0, 0, 2, 0, 0, 1, 1, 1, 0, 1, 0, 4, 4, 4, 4, 4};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nseq;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = offs[i], e = offs[i + 1];
        float c[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        for (uint64_t q = b; q < e; ++q) {
            const uint8_t r = seq[q];
            c[r < 25 ? grp[r] : 4] += 1.f;
        }
        const float inv = e > b ? 1.f / (float)(e - b) : 0.f;
        comp[i] = make_float4(c[0] * inv, c[1] * inv, c[2] * inv, c[3] * inv);
    }
}

constexpr int WIN_BEFORE = 32, WIN_LEN = 64;

__device__ float diag_window(const uint8_t *V, int m, const uint8_t *H, int n, int r0, int c0,
                             const int8_t *sm)
{
    int s = 0, cnt = 0;
    for (int t = -WIN_BEFORE; t < WIN_LEN - WIN_BEFORE; ++t) {
        const int i = r0 + t, j = c0 + t;
        if (i < 0 || j < 0 || i >= m || j >= n) continue;
        s += sm[V[i] * PG_NRES + H[j]];
        ++cnt;
    }
    return cnt ? (float)s / (4.f * (float)cnt) : 0.f;
}

__global__ void k_features(const pg_pair *pairs, uint64_t n, uint64_t roff, uint64_t coff,
                           const uint8_t *rseq, const uint64_t *roffs, uint64_t nr,
                           const uint8_t *cseq, const uint64_t *coffs, uint64_t nc,
                           const int8_t *sm, const float4 *rcomp, const float4 *ccomp,
                           __nv_bfloat16 *X, int *status)
{
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const pg_pair pr = pairs[p];
        const uint64_t r = pr.row + roff, c = pr.col + coff;
        float f[NF];
        if (r >= nr || c >= nc) {
            atomicOr(status, 1);
            for (int k = 0; k < NF; ++k) f[k] = 0.f;
        } else {
            const float m = (float)(roffs[r + 1] - roffs[r]), nn = (float)(coffs[c + 1] - coffs[c]);
            const float mm = fmaxf(m, 1.f), n1 = fmaxf(nn, 1.f), L = fmaxf(mm, n1);
            const bool two = pr.count >= 2;
            const float d0 = ((float)pr.cs0 - (float)pr.rs0) / L;
            const float d1 = ((float)pr.cs1 - (float)pr.rs1) / L;
            f[0] = log2f(1.f + (float)pr.count) * 0.25f;
            f[1] = (float)pr.score * (1.f / 32.f);
            f[2] = two ? 1.f : 0.f;
            f[3] = d0;
            f[4] = two ? d1 : 0.f;
            f[5] = two ? fabsf(d0 - d1) : 0.f;
            f[6] = (float)pr.rs0 / mm;
            f[7] = (float)pr.cs0 / n1;
            {
                const uint8_t *V = rseq + roffs[r], *H = cseq + coffs[c];
                const int mi = (int)(roffs[r + 1] - roffs[r]), ni = (int)(coffs[c + 1] - coffs[c]);
                float w = diag_window(V, mi, H, ni, pr.rs0, pr.cs0, sm);
                if (two && (pr.rs1 != pr.rs0 || pr.cs1 != pr.cs0))
                    w = fmaxf(w, diag_window(V, mi, H, ni, pr.rs1, pr.cs1, sm));
                f[8] = w;
            }
            f[9] = log2f(mm) * (1.f / 12.f);
            f[10] = log2f(n1) * (1.f / 12.f);
            f[11] = fabsf(log2f(mm / n1));
            const float4 a = rcomp[r], b = ccomp[c];
            f[12] = fabsf(a.x - b.x);
            f[13] = fabsf(a.y - b.y);
            f[14] = fabsf(a.z - b.z);
            f[15] = fabsf(a.w - b.w);
        }
        __nv_bfloat16 *o = X + p * NF;
#pragma unroll
        for (int k = 0; k < NF; k += 2) {
            *reinterpret_cast<__nv_bfloat162 *>(o + k) = __floats2bfloat162_rn(f[k], f[k + 1]);
        }
    }
}

__global__ void __launch_bounds__(FWARPS * 32) k_mlp_forward(const float *P, const __nv_bfloat16 *X,
                                                              uint64_t n, float *logits)
{
    __shared__ SmemW s;
    load_weights(s, P);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint64_t tiles = (n + 15) / 16;
    for (uint64_t tile = blockIdx.x * (uint64_t)FWARPS + (threadIdx.x >> 5); tile < tiles;
         tile += (uint64_t)gridDim.x * FWARPS) {
        Tile T;
        forward_tile(s, X, n, tile * 16, T);
        if (t == 0) {
            const uint64_t r0 = tile * 16 + g, r1 = r0 + 8;
            if (r0 < n) logits[r0] = T.z0;
            if (r1 < n) logits[r1] = T.z1;
        }
    }
}

// Per-warp staging for the weight-gradient GEMMs (all [row][sample], bf16)
struct WarpStage {
    __nv_bfloat16 dh2t[NH * 16];   // dL/d(pre-activation 2), [unit][sample]
    __nv_bfloat16 h1t[NH * 16];    // h1 as layer 2 saw it, [unit][sample]
    __nv_bfloat16 dh1t[NH * 16];   // dL/d(pre-activation 1), [unit][sample]
    __nv_bfloat16 xt[NF * 16];     // x, [feature][sample]
};

struct GradAcc {
    float w1t[NH * NF], b1[NH], w2t[NH * NH], b2[NH], w3[NH], b3, loss;
};

// One pass over a mini-batch: forward, binary cross-entropy with logits
// (weighted by wts, averaged by inv_norm), backward, and gradient
// accumulation into G (same layout as P) and *loss.
__global__ void __launch_bounds__(FWARPS * 32) k_mlp_backward(const float *P, const __nv_bfloat16 *X,
                                                               const float *label, const float *wts,
                                                               uint64_t n, float inv_norm, float *G)
{
    extern __shared__ unsigned char fsm[];
    SmemW &s = *reinterpret_cast<SmemW *>(fsm);
    GradAcc &acc = *reinterpret_cast<GradAcc *>(fsm + sizeof(SmemW));
    WarpStage *stages = reinterpret_cast<WarpStage *>(fsm + sizeof(SmemW) + sizeof(GradAcc));
    load_weights(s, P);
    {
        float *a = reinterpret_cast<float *>(&acc);
        for (int k = threadIdx.x; k < (int)(sizeof(GradAcc) / sizeof(float)); k += blockDim.x) a[k] = 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, wib = threadIdx.x >> 5;
    WarpStage &st = stages[wib];
    const uint64_t tiles = (n + 15) / 16;
    for (uint64_t tile = blockIdx.x * (uint64_t)FWARPS + wib; tile < tiles;
         tile += (uint64_t)gridDim.x * FWARPS) {
        const uint64_t base = tile * 16;
        Tile T;
        forward_tile(s, X, n, base, T);
        const uint64_t r0 = base + g, r1 = r0 + 8;
        const float y0 = r0 < n ? label[r0] : 0.f, y1 = r1 < n ? label[r1] : 0.f;
        const float w0 = r0 < n ? wts[r0] : 0.f, w1 = r1 < n ? wts[r1] : 0.f;
        const float p0 = 1.f / (1.f + __expf(-T.z0)), p1 = 1.f / (1.f + __expf(-T.z1));
        const float dz0 = w0 * (p0 - y0) * inv_norm, dz1 = w1 * (p1 - y1) * inv_norm;
        if (t == 0) {
            const float l0 = fmaxf(T.z0, 0.f) - T.z0 * y0 + log1pf(__expf(-fabsf(T.z0)));
            const float l1 = fmaxf(T.z1, 0.f) - T.z1 * y1 + log1pf(__expf(-fabsf(T.z1)));
            atomicAdd(&acc.loss, (w0 * l0 + w1 * l1) * inv_norm);
            atomicAdd(&acc.b3, dz0 + dz1);
        }
        // layer 3 and the pre-activation gradient of layer 2
        float dh2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = nt * 8 + 2 * t;
            float gw0 = dz0 * T.h2[nt][0] + dz1 * T.h2[nt][2];
            float gw1 = dz0 * T.h2[nt][1] + dz1 * T.h2[nt][3];
            dh2[nt][0] = T.h2[nt][0] > 0.f ? dz0 * s.w3[c] : 0.f;
            dh2[nt][1] = T.h2[nt][1] > 0.f ? dz0 * s.w3[c + 1] : 0.f;
            dh2[nt][2] = T.h2[nt][2] > 0.f ? dz1 * s.w3[c] : 0.f;
            dh2[nt][3] = T.h2[nt][3] > 0.f ? dz1 * s.w3[c + 1] : 0.f;
            float gb0 = dh2[nt][0] + dh2[nt][2], gb1 = dh2[nt][1] + dh2[nt][3];
            // sum over the 8 row groups (lanes with the same t)
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                gw0 += __shfl_xor_sync(0xffffffffu, gw0, o);
                gw1 += __shfl_xor_sync(0xffffffffu, gw1, o);
                gb0 += __shfl_xor_sync(0xffffffffu, gb0, o);
                gb1 += __shfl_xor_sync(0xffffffffu, gb1, o);
            }
            if (g == 0) {
                atomicAdd(&acc.w3[c], gw0);
                atomicAdd(&acc.w3[c + 1], gw1);
                atomicAdd(&acc.b2[c], gb0);
                atomicAdd(&acc.b2[c + 1], gb1);
            }
        }
        // dh1 = dh2 W2 (tensor cores), masked by the layer-1 ReLU
        uint32_t a[4][4];
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
            a[kc][0] = pack_bf16(dh2[2 * kc][0], dh2[2 * kc][1]);
            a[kc][1] = pack_bf16(dh2[2 * kc][2], dh2[2 * kc][3]);
            a[kc][2] = pack_bf16(dh2[2 * kc + 1][0], dh2[2 * kc + 1][1]);
            a[kc][3] = pack_bf16(dh2[2 * kc + 1][2], dh2[2 * kc + 1][3]);
        }
        float dh1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kc = 0; kc < 4; ++kc) {
                const __nv_bfloat16 *w = s.w2 + (nt * 8 + g) * NH + kc * 16 + 2 * t;
                mma16816(d, a[kc], ld_u32(w), ld_u32(w + 8));
            }
            dh1[nt][0] = T.h1[nt][0] > 0.f ? d[0] : 0.f;
            dh1[nt][1] = T.h1[nt][1] > 0.f ? d[1] : 0.f;
            dh1[nt][2] = T.h1[nt][2] > 0.f ? d[2] : 0.f;
            dh1[nt][3] = T.h1[nt][3] > 0.f ? d[3] : 0.f;
            const int c = nt * 8 + 2 * t;
            float gb0 = dh1[nt][0] + dh1[nt][2], gb1 = dh1[nt][1] + dh1[nt][3];
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                gb0 += __shfl_xor_sync(0xffffffffu, gb0, o);
                gb1 += __shfl_xor_sync(0xffffffffu, gb1, o);
            }
            if (g == 0) {
                atomicAdd(&acc.b1[c], gb0);
                atomicAdd(&acc.b1[c + 1], gb1);
            }
        }
        // stage the transposed operands of the weight-gradient GEMMs
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = nt * 8 + 2 * t;
            st.dh2t[c * 16 + g] = __float2bfloat16_rn(dh2[nt][0]);
            st.dh2t[(c + 1) * 16 + g] = __float2bfloat16_rn(dh2[nt][1]);
            st.dh2t[c * 16 + g + 8] = __float2bfloat16_rn(dh2[nt][2]);
            st.dh2t[(c + 1) * 16 + g + 8] = __float2bfloat16_rn(dh2[nt][3]);
            st.h1t[c * 16 + g] = __float2bfloat16_rn(T.h1[nt][0]);
            st.h1t[(c + 1) * 16 + g] = __float2bfloat16_rn(T.h1[nt][1]);
            st.h1t[c * 16 + g + 8] = __float2bfloat16_rn(T.h1[nt][2]);
            st.h1t[(c + 1) * 16 + g + 8] = __float2bfloat16_rn(T.h1[nt][3]);
            st.dh1t[c * 16 + g] = __float2bfloat16_rn(dh1[nt][0]);
            st.dh1t[(c + 1) * 16 + g] = __float2bfloat16_rn(dh1[nt][1]);
            st.dh1t[c * 16 + g + 8] = __float2bfloat16_rn(dh1[nt][2]);
            st.dh1t[(c + 1) * 16 + g + 8] = __float2bfloat16_rn(dh1[nt][3]);
        }
        for (int k = lane; k < NF * 16; k += 32) {
            const int f = k / 16, smp = k % 16;
            const uint64_t r = base + smp;
            st.xt[k] = r < n ? X[r * NF + f] : __float2bfloat16_rn(0.f);
        }
        __syncwarp();
        // dW2[o][i] = sum_s dh2[s][o] h1[s][i]:  M = o, N = i, K = the 16 samples
#pragma unroll
        for (int mt = 0; mt < 4; ++mt) {
            uint32_t am[4];
            am[0] = ld_u32(st.dh2t + (mt * 16 + g) * 16 + 2 * t);
            am[1] = ld_u32(st.dh2t + (mt * 16 + g + 8) * 16 + 2 * t);
            am[2] = ld_u32(st.dh2t + (mt * 16 + g) * 16 + 2 * t + 8);
            am[3] = ld_u32(st.dh2t + (mt * 16 + g + 8) * 16 + 2 * t + 8);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                const __nv_bfloat16 *b = st.h1t + (nt * 8 + g) * 16 + 2 * t;
                mma16816(d, am, ld_u32(b), ld_u32(b + 8));
                const int o0 = mt * 16 + g, i0 = nt * 8 + 2 * t;
                atomicAdd(&acc.w2t[o0 * NH + i0], d[0]);
                atomicAdd(&acc.w2t[o0 * NH + i0 + 1], d[1]);
                atomicAdd(&acc.w2t[(o0 + 8) * NH + i0], d[2]);
                atomicAdd(&acc.w2t[(o0 + 8) * NH + i0 + 1], d[3]);
            }
        }
        // dW1[o][f] = sum_s dh1[s][o] x[s][f]:  M = o, N = f, K = samples
#pragma unroll
        for (int mt = 0; mt < 4; ++mt) {
            uint32_t am[4];
            am[0] = ld_u32(st.dh1t + (mt * 16 + g) * 16 + 2 * t);
            am[1] = ld_u32(st.dh1t + (mt * 16 + g + 8) * 16 + 2 * t);
            am[2] = ld_u32(st.dh1t + (mt * 16 + g) * 16 + 2 * t + 8);
            am[3] = ld_u32(st.dh1t + (mt * 16 + g + 8) * 16 + 2 * t + 8);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                const __nv_bfloat16 *b = st.xt + (nt * 8 + g) * 16 + 2 * t;
                mma16816(d, am, ld_u32(b), ld_u32(b + 8));
                const int o0 = mt * 16 + g, f0 = nt * 8 + 2 * t;
                atomicAdd(&acc.w1t[o0 * NF + f0], d[0]);
                atomicAdd(&acc.w1t[o0 * NF + f0 + 1], d[1]);
                atomicAdd(&acc.w1t[(o0 + 8) * NF + f0], d[2]);
                atomicAdd(&acc.w1t[(o0 + 8) * NF + f0 + 1], d[3]);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int k = threadIdx.x; k < NH * NF; k += blockDim.x) atomicAdd(&G[P_W1 + k], acc.w1t[k]);
    for (int k = threadIdx.x; k < NH * NH; k += blockDim.x) atomicAdd(&G[P_W2 + k], acc.w2t[k]);
    for (int k = threadIdx.x; k < NH; k += blockDim.x) {
        atomicAdd(&G[P_B1 + k], acc.b1[k]);
        atomicAdd(&G[P_B2 + k], acc.b2[k]);
        atomicAdd(&G[P_W3 + k], acc.w3[k]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&G[P_B3], acc.b3);
        atomicAdd(&G[NPARAM], acc.loss);
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master copy; clears the gradients.
__global__ void k_adam(float *P, float *G, float *M1, float *M2, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NPARAM) return;
    const float gk = G[k];
    const float m = b1 * M1[k] + (1.f - b1) * gk;
    const float v = b2 * M2[k] + (1.f - b2) * gk * gk;
    M1[k] = m;
    M2[k] = v;
    P[k] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    G[k] = 0.f;
}

__global__ void k_compact(const float *logits, uint64_t n, float thr, unsigned int *count,
                          uint32_t *kept_idx)
{
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        if (logits[p] >= thr) {
            const unsigned int slot = atomicAdd(count, 1u);
            kept_idx[slot] = (uint32_t)p;
        }
    }
}

__global__ void k_gather(const pg_pair *pairs, const uint32_t *kept_idx, const unsigned int *count,
                         pg_pair *out)
{
    const unsigned int n = *count;
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
        out[q] = pairs[kept_idx[q]];
}

// pruned pairs get an empty result with PG_RF_FILTERED; kept ones their alignment
__global__ void k_scatter(const pg_result *kept_res, const uint32_t *kept_idx, const unsigned int *count,
                          const float *logits, uint64_t n, float thr, pg_result *out)
{
    const unsigned int nk = *count;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        if (logits[p] < thr) {
            pg_result o;
            o.score = 0; o.aln_len = 0; o.matches = 0; o.gap_opens = 0;
            o.beg_h = o.end_h = o.beg_v = o.end_v = 0;
            o.identity = 0.f; o.score_aln = 0.f; o.seed_used = 0;
            o.flags = PG_RF_EMPTY | PG_RF_FILTERED; o.pad = 0; o.cells = 0;
            out[p] = o;
        }
    }
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < nk; q += gridDim.x * blockDim.x)
        out[kept_idx[q]] = kept_res[q];
}

size_t backward_smem() { return sizeof(SmemW) + sizeof(GradAcc) + FWARPS * sizeof(WarpStage); }

}  // namespace

struct pg_filter {
    int device = 0;
    float *d_P = nullptr, *d_G = nullptr, *d_M1 = nullptr, *d_M2 = nullptr;  // G has NPARAM+1 (loss)
    int step = 0;
    int nsm = 0;
    // per-call scratch
    float4 *d_rcomp = nullptr, *d_ccomp = nullptr;
    uint64_t comp_cap_r = 0, comp_cap_c = 0;
    __nv_bfloat16 *d_X = nullptr;
    float *d_logit = nullptr;
    uint32_t *d_idx = nullptr;
    unsigned int *d_cnt = nullptr;
    pg_pair *d_kept = nullptr;
    pg_result *d_kres = nullptr;
    int *d_status = nullptr;
    uint64_t cap = 0;
};

extern "C" {

int pg_filter_create(int device, uint64_t seed, pg_filter **out)
{
    if (!out) return pg_internal_fail(PG_ERR_ARG, "pg_filter_create: null output");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return pg_internal_fail(PG_ERR_NODEV, "pg_filter_create: no such device");
    FCU(cudaSetDevice(device));
    pg_filter *f = new pg_filter();
    f->device = device;
    cudaDeviceGetAttribute(&f->nsm, cudaDevAttrMultiProcessorCount, device);
    // He-uniform initialisation from a fixed-seed generator (splitmix64)
    std::vector<float> P(NPARAM, 0.f);
    uint64_t x = seed ^ 0x9e3779b97f4a7c15ull;
    auto unif = [&x]() {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    const double a1 = std::sqrt(6.0 / NF), a2 = std::sqrt(6.0 / NH), a3 = std::sqrt(3.0 / NH);
    for (int k = 0; k < NH * NF; ++k) P[P_W1 + k] = (float)(a1 * unif());
    for (int k = 0; k < NH * NH; ++k) P[P_W2 + k] = (float)(a2 * unif());
    for (int k = 0; k < NH; ++k) P[P_W3 + k] = (float)(a3 * unif());
    cudaError_t e = cudaMalloc(&f->d_P, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&f->d_G, (NPARAM + 1) * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&f->d_M1, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&f->d_M2, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&f->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(f->d_P, P.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(f->d_G, 0, (NPARAM + 1) * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(f->d_M1, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(f->d_M2, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)backward_smem());
    if (e != cudaSuccess) {
        pg_filter_destroy(f);
        return pg_internal_fail(e == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA,
                                cudaGetErrorString(e));
    }
    *out = f;
    return PG_OK;
}

void pg_filter_destroy(pg_filter *f)
{
    if (!f) return;
    cudaSetDevice(f->device);
    cudaFree(f->d_P); cudaFree(f->d_G); cudaFree(f->d_M1); cudaFree(f->d_M2);
    cudaFree(f->d_rcomp); cudaFree(f->d_ccomp); cudaFree(f->d_X); cudaFree(f->d_logit);
    cudaFree(f->d_idx); cudaFree(f->d_cnt); cudaFree(f->d_kept); cudaFree(f->d_kres);
    cudaFree(f->d_status);
    delete f;
}

int pg_filter_params(pg_filter *f, float *host, int get)
{
    if (!f || !host) return pg_internal_fail(PG_ERR_ARG, "pg_filter_params: null argument");
    FCU(cudaSetDevice(f->device));
    if (get) FCU(cudaMemcpy(host, f->d_P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    else FCU(cudaMemcpy(f->d_P, host, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    return PG_OK;
}

int pg_filter_features(pg_filter *f, pg_ctx *ctx, const pg_pair *d_pairs, uint64_t n,
                       uint64_t bl_roffset, uint64_t bl_coffset, void *d_features, void *stream)
{
    if (!f || !ctx || (n && (!d_pairs || !d_features)))
        return pg_internal_fail(PG_ERR_ARG, "pg_filter_features: bad argument");
    const uint8_t *rseq, *cseq;
    const uint64_t *roffs, *coffs;
    uint64_t nr, nc;
    int dev, mode;
    void *cst;
    int rc = pg_internal_seqs(ctx, &rseq, &roffs, &nr, &cseq, &coffs, &nc, &dev, &cst, &mode);
    if (rc) return rc;
    const int8_t *d_sm = nullptr;
    rc = pg_internal_score(ctx, &d_sm);
    if (rc) return rc;
    FCU(cudaSetDevice(f->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)cst;
    if (nr > f->comp_cap_r) {
        cudaFree(f->d_rcomp); f->d_rcomp = nullptr; f->comp_cap_r = 0;
        FCU(cudaMalloc(&f->d_rcomp, nr * sizeof(float4)));
        f->comp_cap_r = nr;
    }
    if (nc > f->comp_cap_c) {
        cudaFree(f->d_ccomp); f->d_ccomp = nullptr; f->comp_cap_c = 0;
        FCU(cudaMalloc(&f->d_ccomp, nc * sizeof(float4)));
        f->comp_cap_c = nc;
    }
    const int grid = f->nsm * 8;
    k_composition<<<grid, 256, 0, st>>>(rseq, roffs, nr, f->d_rcomp);
    k_composition<<<grid, 256, 0, st>>>(cseq, coffs, nc, f->d_ccomp);
    FCU(cudaMemsetAsync(f->d_status, 0, sizeof(int), st));
    if (n) k_features<<<grid, 256, 0, st>>>(d_pairs, n, bl_roffset, bl_coffset, rseq, roffs, nr,
                                           cseq, coffs, nc, d_sm, f->d_rcomp, f->d_ccomp,
                                           (__nv_bfloat16 *)d_features, f->d_status);
    FCU(cudaGetLastError());
    int status = 0;
    FCU(cudaMemcpyAsync(&status, f->d_status, sizeof status, cudaMemcpyDeviceToHost, st));
    FCU(cudaStreamSynchronize(st));
    if (status) return pg_internal_fail(PG_ERR_ARG, "pg_filter_features: pair index out of range");
    return PG_OK;
}

int pg_filter_predict(pg_filter *f, const void *d_features, uint64_t n, float *d_logits, void *stream)
{
    if (!f || (n && (!d_features || !d_logits))) return pg_internal_fail(PG_ERR_ARG, "pg_filter_predict: bad argument");
    if (!n) return PG_OK;
    FCU(cudaSetDevice(f->device));
    const uint64_t tiles = (n + 15) / 16;
    const uint64_t blocks = std::min<uint64_t>((tiles + FWARPS - 1) / FWARPS, (uint64_t)f->nsm * 16);
    k_mlp_forward<<<(unsigned)blocks, FWARPS * 32, 0, (cudaStream_t)stream>>>(
        f->d_P, (const __nv_bfloat16 *)d_features, n, d_logits);
    FCU(cudaGetLastError());
    return PG_OK;
}

int pg_filter_gradients(pg_filter *f, const void *d_features, const float *d_labels,
                        const float *d_weights, uint64_t n, float *host_grad_and_loss, void *stream)
{
    if (!f || !n || !d_features || !d_labels || !d_weights)
        return pg_internal_fail(PG_ERR_ARG, "pg_filter_gradients: bad argument");
    FCU(cudaSetDevice(f->device));
    cudaStream_t st = (cudaStream_t)stream;
    FCU(cudaMemsetAsync(f->d_G, 0, (NPARAM + 1) * sizeof(float), st));
    const uint64_t tiles = (n + 15) / 16;
    const uint64_t blocks = std::min<uint64_t>((tiles + FWARPS - 1) / FWARPS, (uint64_t)f->nsm * 4);
    k_mlp_backward<<<(unsigned)blocks, FWARPS * 32, backward_smem(), st>>>(
        f->d_P, (const __nv_bfloat16 *)d_features, d_labels, d_weights, n, 1.0f / (float)n, f->d_G);
    FCU(cudaGetLastError());
    if (host_grad_and_loss) {
        FCU(cudaMemcpyAsync(host_grad_and_loss, f->d_G, (NPARAM + 1) * sizeof(float),
                            cudaMemcpyDeviceToHost, st));
        FCU(cudaStreamSynchronize(st));
    }
    return PG_OK;
}

int pg_filter_train_step(pg_filter *f, const void *d_features, const float *d_labels,
                         const float *d_weights, uint64_t n, float lr, float *loss, void *stream)
{
    int rc = pg_filter_gradients(f, d_features, d_labels, d_weights, n, nullptr, stream);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    float l = 0.f;
    if (loss) FCU(cudaMemcpyAsync(&l, f->d_G + NPARAM, sizeof(float), cudaMemcpyDeviceToHost, st));
    f->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)f->step), c2 = 1.f - std::pow(b2, (float)f->step);
    k_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(f->d_P, f->d_G, f->d_M1, f->d_M2, lr, b1, b2, 1e-8f, c1, c2);
    FCU(cudaGetLastError());
    if (loss) {
        FCU(cudaStreamSynchronize(st));
        *loss = l;
    }
    return PG_OK;
}

int pg_align_filtered(pg_ctx *ctx, pg_filter *f, float threshold, const pg_pair *d_pairs, uint64_t n,
                      uint64_t bl_roffset, uint64_t bl_coffset, pg_result *d_out, void *stream,
                      uint64_t *kept)
{
    if (!ctx || !f || (n && (!d_pairs || !d_out))) return pg_internal_fail(PG_ERR_ARG, "pg_align_filtered: bad argument");
    if (kept) *kept = 0;
    if (!n) return PG_OK;
    FCU(cudaSetDevice(f->device));
    if (n > f->cap) {
        cudaFree(f->d_X); cudaFree(f->d_logit); cudaFree(f->d_idx); cudaFree(f->d_kept); cudaFree(f->d_kres);
        f->d_X = nullptr; f->d_logit = nullptr; f->d_idx = nullptr; f->d_kept = nullptr; f->d_kres = nullptr;
        f->cap = 0;
        FCU(cudaMalloc(&f->d_X, n * NF * sizeof(__nv_bfloat16)));
        FCU(cudaMalloc(&f->d_logit, n * sizeof(float)));
        FCU(cudaMalloc(&f->d_idx, n * sizeof(uint32_t)));
        FCU(cudaMalloc(&f->d_kept, n * sizeof(pg_pair)));
        FCU(cudaMalloc(&f->d_kres, n * sizeof(pg_result)));
        f->cap = n;
    }
    if (!f->d_cnt) FCU(cudaMalloc(&f->d_cnt, sizeof(unsigned int)));
    cudaStream_t st = (cudaStream_t)stream;
    int rc = pg_filter_features(f, ctx, d_pairs, n, bl_roffset, bl_coffset, f->d_X, stream);
    if (rc) return rc;
    rc = pg_filter_predict(f, f->d_X, n, f->d_logit, stream);
    if (rc) return rc;
    FCU(cudaMemsetAsync(f->d_cnt, 0, sizeof(unsigned int), st));
    const int grid = f->nsm * 8;
    k_compact<<<grid, 256, 0, st>>>(f->d_logit, n, threshold, f->d_cnt, f->d_idx);
    k_gather<<<grid, 256, 0, st>>>(d_pairs, f->d_idx, f->d_cnt, f->d_kept);
    unsigned int nk = 0;
    FCU(cudaMemcpyAsync(&nk, f->d_cnt, sizeof nk, cudaMemcpyDeviceToHost, st));
    FCU(cudaStreamSynchronize(st));
    if (nk) {
        rc = pg_align_device(ctx, f->d_kept, nk, bl_roffset, bl_coffset, f->d_kres, stream);
        if (rc) return rc;
    }
    k_scatter<<<grid, 256, 0, st>>>(f->d_kres, f->d_idx, f->d_cnt, f->d_logit, n, threshold, d_out);
    FCU(cudaGetLastError());
    if (kept) *kept = nk;
    return PG_OK;
}

int pg_filter_nparams(void) { return NPARAM; }

}  // extern "C"
