// pg_kernels.cuh -- batch kernels behind pg_align (sm_103a).
//
// Persistent, work-stealing launch: a grid sized to the resident capacity of
// the GPU; each warp takes the next pair index from a device counter until the
// batch is done, so pairs of very different lengths balance themselves.  Each
// pair is finished inside one warp (extension, alignment, statistics, filter),
// so no intermediate result leaves the SM.
#pragma once
#include <cstdint>

#include "../../include/pastis_gb300.h"
#include "pg_dp.cuh"
#include "pg_xdrop.cuh"

namespace pg {

constexpr int WARPS = 8;          // warps per block
constexpr int RING_W = 256;       // shared-memory X-drop ring (ints per anti-diagonal)

// status word bits (read back by the host after a batch)
constexpr int ST_BAD_INDEX = 1;

struct KParams {
    const pg_pair *pairs;
    uint64_t n;
    uint64_t roff, coff;
    const uint8_t *rseq; const uint64_t *roffs; uint64_t nr;
    const uint8_t *cseq; const uint64_t *coffs; uint64_t nc;
    pg_result *out;
    const int8_t *sm;             // 25 x 25
    int go, ge, xg, xdrop, seed_len, seed_count, flags, ani_thr;
    double cov_thr;
    unsigned int *counter;        // work counter (zeroed before launch)
    int *status;                  // error bits
    unsigned long long *exec_cells; // cells actually computed (whole batch)
    Edge *bnd;                    // per-warp row scratch, bnd_stride entries each
    uint64_t bnd_stride;
    int *gring;                   // per-warp fallback ring, 3 * gring_w ints each
    int gring_w;
};

__device__ __forceinline__ void load_sm(int *ssm, const int8_t *sm)
{
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
        const int a = t >> 5, b = t & 31;
        ssm[t] = (a < PG_NRES && b < PG_NRES) ? (int)sm[a * PG_NRES + b] : 0;
    }
}

__device__ __forceinline__ uint32_t sat_u32(uint64_t x) { return x > 0xffffffffull ? 0xffffffffu : (uint32_t)x; }

// identity exactly as computeAlignmentStats forms it, then the coverage/ANI
// filter of SeqanFullAligner.cpp:247-260 / SeqanXdropAligner.cpp:337-352
__device__ __forceinline__ float identity_of(uint32_t M, uint32_t L)
{
    return (float)((100.0 * (double)M) / (double)L);
}

__device__ __forceinline__ void apply_filter(pg_result &o, int len_r, int len_c, double cov_thr, int ani_thr)
{
    const double a = (double)o.aln_len - (double)o.gap_opens;
    const double cc = a / (double)len_c, cr = a / (double)len_r;
    const double cov = cc > cr ? cc : cr;
    if (!(o.flags & PG_RF_EMPTY) && cov >= cov_thr && o.identity >= (float)ani_thr) {
        o.score_aln = o.identity / 100.0f;
        o.flags |= PG_RF_PASSED;
    } else {
        o.score_aln = 0.0f;
    }
}

__device__ __forceinline__ bool fetch_task(const KParams &kp, uint64_t &task)
{
    const int lane = threadIdx.x & 31;
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(kp.counter, 1u);
    t = __shfl_sync(FULL, t, 0);
    task = t;
    return task < kp.n;
}

// resolve a pair's sequences; false (and a status bit) on a bad index
__device__ __forceinline__ bool pair_seqs(const KParams &kp, const pg_pair &pr,
                                          const uint8_t *&V, int &m, const uint8_t *&Hs, int &n)
{
    const uint64_t r = (uint64_t)pr.row + kp.roff, c = (uint64_t)pr.col + kp.coff;
    if (r >= kp.nr || c >= kp.nc) {
        if ((threadIdx.x & 31) == 0) atomicOr(kp.status, ST_BAD_INDEX);
        return false;
    }
    const uint64_t r0 = kp.roffs[r], c0 = kp.coffs[c];
    V = kp.rseq + r0; m = (int)(kp.roffs[r + 1] - r0);
    Hs = kp.cseq + c0; n = (int)(kp.coffs[c + 1] - c0);
    return true;
}

// --------------------------------------------------------------- --sfa (SW)
template <int TIE>
__global__ void __launch_bounds__(WARPS * 32) k_sw(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    Edge *bnd = kp.bnd + gw * kp.bnd_stride;
    unsigned long long exec = 0;
    uint64_t task;
    while (fetch_task(kp, task)) {
        const pg_pair pr = kp.pairs[task];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result o;
        o.score = 0; o.aln_len = 0; o.matches = 0; o.gap_opens = 0;
        o.beg_h = o.end_h = o.beg_v = o.end_v = 0;
        o.identity = 0.0f; o.score_aln = 0.0f; o.seed_used = 0; o.flags = PG_RF_EMPTY;
        o.pad = 0; o.cells = 0;
        if (pair_seqs(kp, pr, V, m, Hs, n)) {
            const DpOut d = dp_dispatch<true, TIE>(V, m, Hs, n, ssm, kp.go, kp.ge, bnd);
            exec += (unsigned long long)m * (unsigned long long)n;
            o.cells = sat_u32((uint64_t)m * (uint64_t)n);
            if (d.have) {
                const uint32_t D = d.st.md >> 16, M = d.st.md & 0xffffu;
                const int i0 = (int)(d.st.b & 0xffffu), j0 = (int)(d.st.b >> 16);
                const uint32_t L = (uint32_t)((d.ei - i0) + (d.ej - j0)) - D;
                o.score = d.score;
                o.aln_len = L; o.matches = M; o.gap_opens = d.st.g;
                o.beg_v = (uint16_t)i0; o.end_v = (uint16_t)d.ei;
                o.beg_h = (uint16_t)j0; o.end_h = (uint16_t)d.ej;
                if (L == 0) { o.identity = 0.0f; }
                else { o.identity = identity_of(M, L); o.flags = 0; }
            }
            apply_filter(o, m, n, kp.cov_thr, kp.ani_thr);
        }
        if (lane == 0) kp.out[task] = o;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells, exec);
}

// --------------------------------------------------------------- --sxa
// one direction of X-drop, shared ring first, per-warp global ring on overflow
__device__ __forceinline__ XdOut xdrop_dir_any(const uint8_t *V, int nv, int vstep,
                                               const uint8_t *Hs, int nh, int hstep,
                                               const int *ssm, int g, int X, int *sring,
                                               int *gring, int gring_w)
{
    XdOut o = xdrop_dir_warp(V, nv, vstep, Hs, nh, hstep, ssm, g, X, sring, RING_W);
    if (!o.ok) o = xdrop_dir_warp(V, nv, vstep, Hs, nh, hstep, ssm, g, X, gring, gring_w);
    return o;
}

template <int TIE>
__global__ void __launch_bounds__(WARPS * 32) k_xdrop(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    __shared__ int sring[WARPS][3 * RING_W];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + wib;
    Edge *bnd = kp.bnd + gw * kp.bnd_stride;
    int *gring = kp.gring + gw * 3ull * (uint64_t)kp.gring_w;
    int *ring = sring[wib];
    unsigned long long exec = 0;
    uint64_t task;
    while (fetch_task(kp, task)) {
        const pg_pair pr = kp.pairs[task];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result best;
        best.score = 0; best.aln_len = 0; best.matches = 0; best.gap_opens = 0;
        best.beg_h = best.end_h = best.beg_v = best.end_v = 0;
        best.identity = 0.0f; best.score_aln = 0.0f; best.seed_used = 0;
        best.flags = PG_RF_EMPTY; best.pad = 0; best.cells = 0;
        if (pair_seqs(kp, pr, V, m, Hs, n)) {
            uint64_t cells = 0;
            bool have = false, badseed = false;
            int prev_r0 = -1, prev_c0 = -1, pbv = 0, pev = 0, pbh = 0, peh = 0;
            uint32_t prev_xcells = 0;
            for (int cnt = 0; cnt < kp.seed_count && cnt < 2; ++cnt) {
                if (cnt > 0 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && pr.count < 2) break;
                const int r0 = cnt == 0 ? pr.rs0 : pr.rs1;
                const int c0 = cnt == 0 ? pr.cs0 : pr.cs1;
                int bv = r0, ev = r0 + kp.seed_len, bh = c0, eh = c0 + kp.seed_len;
                if (ev > m || eh > n) {
                    badseed = true;
                    bv = min(bv, m); ev = min(ev, m); bh = min(bh, n); eh = min(eh, n);
                }
                uint32_t xcells = 0;
                if (cnt > 0 && r0 == prev_r0 && c0 == prev_c0) {
                    // the same seed again: same extension, same alignment; an
                    // equal identity never replaces the kept one
                    cells += prev_xcells + (uint64_t)(pev - pbv) * (uint64_t)(peh - pbh);
                    continue;
                }
                if (bv > 0 && bh > 0) {
                    XdOut x = xdrop_dir_any(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1, ssm, kp.xg,
                                            kp.xdrop, ring, gring, kp.gring_w);
                    xcells += x.cells;
                    bv -= x.dv; bh -= x.dh;
                }
                if (ev < m && eh < n) {
                    XdOut x = xdrop_dir_any(V + ev, m - ev, 1, Hs + eh, n - eh, 1, ssm, kp.xg,
                                            kp.xdrop, ring, gring, kp.gring_w);
                    xcells += x.cells;
                    ev += x.dv; eh += x.dh;
                }
                exec += xcells;
                const uint64_t area = (uint64_t)(ev - bv) * (uint64_t)(eh - bh);
                cells += xcells + area;
                const bool same_region = cnt > 0 && bv == pbv && ev == pev && bh == pbh && eh == peh;
                prev_r0 = r0; prev_c0 = c0; prev_xcells = xcells;
                pbv = bv; pev = ev; pbh = bh; peh = eh;
                if (same_region) continue;   // identical alignment, cannot win
                const DpOut d = dp_dispatch<false, TIE>(V + bv, ev - bv, Hs + bh, eh - bh, ssm,
                                                        kp.go, kp.ge, bnd);
                exec += area;
                const uint32_t D = d.st.md >> 16, M = d.st.md & 0xffffu;
                const uint32_t L = (uint32_t)((ev - bv) + (eh - bh)) - D;
                pg_result cur;
                cur.score = d.score; cur.aln_len = L; cur.matches = M; cur.gap_opens = d.st.g;
                cur.beg_v = (uint16_t)bv; cur.end_v = (uint16_t)ev;
                cur.beg_h = (uint16_t)bh; cur.end_h = (uint16_t)eh;
                cur.seed_used = (uint8_t)cnt; cur.pad = 0; cur.cells = 0; cur.score_aln = 0.0f;
                if (L == 0) { cur.identity = 0.0f; cur.flags = PG_RF_EMPTY; }
                else { cur.identity = identity_of(M, L); cur.flags = 0; }
                // an empty alignment (identity 0/0) never replaces or is replaced
                const bool cur_nan = (cur.flags & PG_RF_EMPTY) != 0;
                const bool best_nan = (best.flags & PG_RF_EMPTY) != 0;
                if (!have || (!cur_nan && !best_nan && cur.identity > best.identity)) {
                    best = cur;
                    have = true;
                }
            }
            best.cells = sat_u32(cells);
            if (badseed) best.flags |= PG_RF_BAD_SEED;
            apply_filter(best, m, n, kp.cov_thr, kp.ani_thr);
        }
        if (lane == 0) kp.out[task] = best;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells, exec);
}

}  // namespace pg
