// pg_kernels.cuh -- batch kernels behind pg_align (sm_103a).
//
// --sxa (X-drop), five launches per batch:
//   k_xdf      one thread per (pair, seed): both X-drop directions on a
//              16-slot per-thread ring in shared memory (the band of the
//              default gap model, with its two border columns, never spans more
//              than 15 columns), stepped
//              one direction at a time; threads take the next (pair, seed)
//              from a device counter the moment a direction ends, so long
//              and short extensions balance.  Writes the extended region.
//   k_xd_wide  one warp per (pair, seed) whose band outgrew the thread ring:
//              256-slot shared ring, per-warp global ring beyond that.
//              (k_xd16, a 16-bit-lane form of the extension, is a tuning option.)
//   k_hist, k_bucket  the bucket order of the pairs for k_ga (schedule below).
//   k_ga       one warp per pair: global alignment with statistics over each
//              seed's region (a region equal to the first seed's is not
//              realigned: an equal identity never replaces the kept one),
//              best identity, coverage/ANI filter, result record.
// --sfa (SW): k_hist, k_bucket, then k_sw, one warp per pair, local
// alignment with statistics.
//
// This file holds the shared parameters and helpers, the schedule and the
// statistics kernels k_ga / k_sw; the extension kernels are in
// pg_kernels_xd.cuh, the traceback form of the alignment in
// pg_kernels_dir.cuh (its own translation unit, pg_dir.cu).
//
// All kernels are persistent with work stealing (grids sized to the resident
// capacity) so pairs of very different lengths balance themselves.
#pragma once
#include <cstdint>

#include "../../include/pastis_gb300.h"
#include "pg_dp.cuh"
#include "pg_dpdir16.cuh"
#include "pg_xdrop.cuh"

namespace pg {

constexpr int WARPS = 8;          // warps per block (k_ga, k_sw, k_xd_wide)
constexpr int RING_W = 256;       // shared ring per warp in k_xd_wide
constexpr int XDA_ARRAYS = 8;     // ring arrays per warp in k_xda (T x 3, E x 2, F x 2)
constexpr int XT = 128;           // threads per block in k_xdf / k_xd16
constexpr int XW = 16;            // per-thread ring slots in k_xdf

// status word bits (read back by the host after a batch)
constexpr int ST_BAD_INDEX = 1;
constexpr int ST_TOO_LONG = 2;    // a sequence beyond a kernel's length bound
constexpr int ST_BAD_SCHED = 4;   // bucket order inconsistent (never expected)
constexpr int ST_BAD_CODE = 8;    // a residue code outside 0..24

// extension of one (pair, seed)
constexpr uint32_t XF_NONE = 1;    // seed not tried (seed_count / spurious switch)
constexpr uint32_t XF_SAME = 2;    // same seed as the first one
constexpr uint32_t XF_BAD = 4;     // seed clamped at a sequence end
constexpr uint32_t XF_OVF = 8;     // band outgrew the thread ring: redo in k_xd_wide
constexpr uint32_t XF_BADIDX = 16; // pair index out of range

struct XdRec {
    uint16_t bv, ev, bh, eh;
    uint32_t cells;
    uint32_t flags;
};

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
    unsigned int *counter;        // [0] k_ga / k_sw pairs, [1] k_xdf tasks, [2] overflow count
    int *status;                  // error bits
    unsigned long long *exec_cells; // cells actually computed: [0] X-drop bands, [1] DP
    XdRec *xd;                    // 2 per pair
    uint32_t *ovf;                // overflowed (pair, seed) tasks
    void *bnd;                    // per-warp row scratch
    uint64_t bnd_bytes;           // bytes per warp
    int *gring;                   // per-warp fallback ring, 3 * gring_w ints each
    int gring_w;
    unsigned int *sched = nullptr;   // [0, NBUCKET) bucket sizes, [NBUCKET, 2*NBUCKET) cursors
    const uint32_t *order = nullptr; // pair taken as the t-th task by k_ga / k_sw (null: t)
    int rows_cap = 8;                // cap on DP rows per lane (tuning)
    int dir = 0;                     // 1: the traceback form (pg_kernels_dir.cuh) runs the DP
    int dir16_lim = 0;               // traceback form: regions with m + n <= this on 16-bit lanes
    int dir16_side = 0;              // ... and larger ones with both sides <= this, checked
    int dir16_pair = 0;              // 1: 16-bit regions of up to 32 x rows_cap rows two per warp
    const uint32_t *xorder = nullptr; // X-drop extension tasks, longest length bound first (null: t)
    unsigned int *xsched = nullptr;   // [0, XBUCKET) task bucket sizes, [XBUCKET, 2*XBUCKET) cursors
};

__device__ __forceinline__ void load_sm(int *ssm, const int8_t *sm)
{
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
        const int a = t >> 5, b = t & 31;
        ssm[t] = (a < PG_NRES && b < PG_NRES) ? (int)sm[a * PG_NRES + b] : 0;
    }
}

__device__ __forceinline__ uint32_t sat_u32(uint64_t x) { return x > 0xffffffffull ? 0xffffffffu : (uint32_t)x; }

// identity exactly as computeAlignmentStats forms it
__device__ __forceinline__ float identity_of(uint32_t M, uint32_t L)
{
    return (float)((100.0 * (double)M) / (double)L);
}

// coverage/ANI filter of SeqanFullAligner.cpp:247-260 / SeqanXdropAligner.cpp:337-352
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

__device__ __forceinline__ pg_result empty_result()
{
    pg_result o;
    o.score = 0; o.aln_len = 0; o.matches = 0; o.gap_opens = 0;
    o.beg_h = o.end_h = o.beg_v = o.end_v = 0;
    o.identity = 0.0f; o.score_aln = 0.0f; o.seed_used = 0; o.flags = PG_RF_EMPTY;
    o.pad = 0; o.cells = 0;
    return o;
}

// Work stealing: one atomic on the shared counter hands a warp FETCH_CHUNK
// consecutive pairs (1: measured no faster with 4, and single pairs balance best).
constexpr unsigned FETCH_CHUNK = 1;

struct WarpQueue {
    uint64_t next = 0, end = 0;
    __device__ __forceinline__ bool pop(unsigned int *counter, uint64_t n, uint64_t &task)
    {
        if (next >= end) {
            unsigned int t = 0;
            if ((threadIdx.x & 31) == 0) t = atomicAdd(counter, FETCH_CHUNK);
            t = __shfl_sync(FULL, t, 0);
            next = t;
            end = (uint64_t)t + FETCH_CHUNK < n ? (uint64_t)t + FETCH_CHUNK : n;
        }
        if (next >= n) return false;
        task = next++;
        return true;
    }
};

// a pair's sequences; false on a bad index
__device__ __forceinline__ bool pair_seqs(const KParams &kp, const pg_pair &pr,
                                          const uint8_t *&V, int &m, const uint8_t *&Hs, int &n)
{
    const uint64_t r = (uint64_t)pr.row + kp.roff, c = (uint64_t)pr.col + kp.coff;
    if (r >= kp.nr || c >= kp.nc) return false;
    const uint64_t r0 = kp.roffs[r], c0 = kp.coffs[c];
    V = kp.rseq + r0; m = (int)(kp.roffs[r + 1] - r0);
    Hs = kp.cseq + c0; n = (int)(kp.coffs[c + 1] - c0);
    return true;
}

// seed s of a pair as a region [bv, ev) x [bh, eh), clamped at sequence ends
__device__ __forceinline__ bool seed_region(const KParams &kp, const pg_pair &pr, int s, int m, int n,
                                            int &bv, int &ev, int &bh, int &eh)
{
    const int r0 = s == 0 ? pr.rs0 : pr.rs1;
    const int c0 = s == 0 ? pr.cs0 : pr.cs1;
    bv = r0; ev = r0 + kp.seed_len; bh = c0; eh = c0 + kp.seed_len;
    if (ev > m || eh > n) {
        bv = min(bv, m); ev = min(ev, m); bh = min(bh, n); eh = min(eh, n);
        return true;
    }
    return false;
}

// ------------------------------------------------------------------ k_ga
// Rows per lane by region height.  A stripe of 32*R rows costs (n + last
// busy lane) column steps of R cells whatever number of its lanes hold rows,
// so the region takes the fewest stripes of at most 32*RMAX rows and spreads
// its rows evenly over them (m = 300: two stripes of R = 5, not 256 + 44 rows
// at R = 8).  One-word statistics go up to 8 rows per lane, the wider ones
// stop at 4 to stay within the register budget.
template <class S>
__host__ __device__ constexpr int dp_rows_max() { return sizeof(S) > 4 ? 4 : 8; }

template <class S>
__host__ __device__ __forceinline__ int dp_rows_per_lane(int m, int cap = 8)
{
    const int RMAX = cap < dp_rows_max<S>() ? (cap < 1 ? 1 : cap) : dp_rows_max<S>();
    const int stripes = m > 0 ? (m + 32 * RMAX - 1) / (32 * RMAX) : 1;
    const int r = (m + 32 * stripes - 1) / (32 * stripes);
    return r < 1 ? 1 : r;
}

template <class S, int TIE>
__device__ __forceinline__ DpOut<S> dp_dispatch(const uint8_t *V, int m, const uint8_t *Hs, int n,
                                                const int *ssm, uint2 *prof, int go, int ge, void *bnd,
                                                int cap = 8)
{
    Edge<S> *b = (Edge<S> *)bnd;
    constexpr int RM = dp_rows_max<S>();
    switch (dp_rows_per_lane<S>(m, cap)) {
    case 1: return dp_warp<S, TIE, 1>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 2: return dp_warp<S, TIE, 2>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 3: return dp_warp<S, TIE, 3>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 4: return dp_warp<S, TIE, 4>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 5: return dp_warp<S, TIE, (RM < 5 ? RM : 5)>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 6: return dp_warp<S, TIE, (RM < 6 ? RM : 6)>(V, m, Hs, n, ssm, prof, go, ge, b);
    case 7: return dp_warp<S, TIE, (RM < 7 ? RM : 7)>(V, m, Hs, n, ssm, prof, go, ge, b);
    default: return dp_warp<S, TIE, RM>(V, m, Hs, n, ssm, prof, go, ge, b);
    }
}

// ------------------------------------------------------------- schedule
// k_ga / k_sw take their pairs in bucket order, one bucket per DP
// instantiation (statistics width x rows per lane), widest and tallest first.
// The warps of an SM then run the same one or two inner loops at a time: all
// instantiations together are larger than the instruction cache, and mixing
// them measured 1.4x slower.  Costly pairs also start first, so cheap ones
// fill the tail of the batch.
constexpr int NBUCKET = 24;
constexpr int SCHED_WORDS = 2 * NBUCKET;
constexpr int XBUCKET = 72;          // extension task buckets: quarter octaves of the length bound
constexpr int XSCHED_WORDS = 2 * XBUCKET;
constexpr int BUCKET_NONE = 23;   // no DP work

// traceback form, lanes of a region's DP (pg_dpdir16.cuh): 0 32-bit; 1 16-bit,
// every value provably inside int16; 2 16-bit, checked, redone on 32-bit lanes
// if a value leaves the range (its borders fit: both sides <= dir16_side).
// (Keeping regions of up to 64 or 128 rows on 32-bit lanes measured no faster.)
__host__ __device__ __forceinline__ int dir16_mode(const KParams &kp, int m, int n)
{
    if (m <= 0 || n <= 0 || kp.dir16_lim <= 0) return 0;
    if (m + n <= kp.dir16_lim) return 1;
    return (m <= kp.dir16_side && n <= kp.dir16_side) ? 2 : 0;
}
__host__ __device__ __forceinline__ bool dir16_use(const KParams &kp, int m, int n)
{
    return dir16_mode(kp, m, n) != 0;
}

// a region whose DP runs on half a warp, two regions per warp (dp_pair_dir16):
// every value provably inside int16 and one stripe of 32 x rows_cap rows
__host__ __device__ __forceinline__ bool dir16_paired(const KParams &kp, int m, int n)
{
    const int cap = kp.rows_cap < 8 ? kp.rows_cap : 8;
    return kp.dir16_pair && dir16_mode(kp, m, n) == 1 && m <= 32 * cap;
}

// traceback form: rows per lane of the region's DP, 16-bit lanes (12..19) after
// 32-bit (4..11); with two regions per warp, the half-warp regions by their
// rows per lane (12..19) and the rest of the 16-bit ones first (0..3)
__device__ __forceinline__ int dir_bucket(const KParams &kp, int m, int n)
{
    if (dir16_use(kp, m, n)) {
        if (!kp.dir16_pair) return 20 - dir16_rows(m, kp.rows_cap);
        if (dir16_paired(kp, m, n)) return 20 - dir16_pair_rows(m);
        return max(0, 8 - dir16_rows(m, kp.rows_cap));
    }
    return 12 - dp_rows_per_lane<S1>(m, kp.rows_cap);
}

// bucket of the first seed's region (X-drop) or of the pair (SW)
template <bool XDROP>
__device__ __forceinline__ int pair_bucket(const KParams &kp, uint64_t p)
{
    int m, n;
    if (XDROP) {
        const XdRec r = kp.xd[2 * p];
        if (r.flags & (XF_NONE | XF_BADIDX)) return BUCKET_NONE;
        m = r.ev - r.bv;
        n = r.eh - r.bh;
        if (m <= 0 || n <= 0) return BUCKET_NONE;
        // the traceback form has no statistics words: one family up to 8 rows
        if (kp.dir) return dir_bucket(kp, m, n);                                                     // 4..19
        if (m > S1::MAXSIDE || n > S1::MAXSIDE) return 4 - dp_rows_per_lane<S2>(m, kp.rows_cap);   // 0..3
        return 12 - dp_rows_per_lane<S1>(m, kp.rows_cap);                                           // 4..11
    }
    const pg_pair pr = kp.pairs[p];
    const uint8_t *V, *Hs;
    if (!pair_seqs(kp, pr, V, m, Hs, n) || m == 0 || n == 0) return BUCKET_NONE;
    if (kp.dir) return dir_bucket(kp, m, n);                                                          // 4..19
    if (m > L1::MAXSIDE || n > L1::MAXSIDE) return 4 - dp_rows_per_lane<L2>(m, kp.rows_cap);        // 0..3
    return 8 - dp_rows_per_lane<L1>(m, kp.rows_cap);                                                // 4..7
}

// bucket sizes
template <bool XDROP>
__global__ void __launch_bounds__(256) k_hist(const KParams kp)
{
    __shared__ unsigned int h[NBUCKET];
    if (threadIdx.x < NBUCKET) h[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < kp.n;
         p += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[pair_bucket<XDROP>(kp, p)], 1u);
    __syncthreads();
    if (threadIdx.x < NBUCKET && h[threadIdx.x]) atomicAdd(&kp.sched[threadIdx.x], h[threadIdx.x]);
}

// order[]: pairs grouped by bucket (any order inside a bucket)
template <bool XDROP>
__global__ void __launch_bounds__(256) k_bucket(const KParams kp)
{
    __shared__ unsigned int start[NBUCKET], h[NBUCKET], base[NBUCKET];
    if (threadIdx.x == 0) {
        unsigned int acc = 0;
        for (int b = 0; b < NBUCKET; ++b) { start[b] = acc; acc += kp.sched[b]; }
    }
    uint32_t *order = const_cast<uint32_t *>(kp.order);
    for (uint64_t c0 = (uint64_t)blockIdx.x * blockDim.x; c0 < kp.n; c0 += (uint64_t)gridDim.x * blockDim.x) {
        if (threadIdx.x < NBUCKET) h[threadIdx.x] = 0;
        __syncthreads();
        const uint64_t p = c0 + threadIdx.x;
        int b = 0;
        unsigned int rank = 0;
        if (p < kp.n) {
            b = pair_bucket<XDROP>(kp, p);
            rank = atomicAdd(&h[b], 1u);
        }
        __syncthreads();
        if (threadIdx.x < NBUCKET && h[threadIdx.x])
            base[threadIdx.x] = start[threadIdx.x] + atomicAdd(&kp.sched[NBUCKET + threadIdx.x], h[threadIdx.x]);
        __syncthreads();
        if (p < kp.n) {
            const uint64_t pos = (uint64_t)base[b] + rank;
            if (pos < kp.n) order[pos] = (uint32_t)p;
            else atomicOr(kp.status, ST_BAD_SCHED);
        }
        __syncthreads();
    }
}

// dynamic shared memory of the warp-per-pair kernels: one score profile per warp
constexpr int DP_DYN_SMEM = WARPS * PROF_BYTES;
constexpr int DIR16_DYN_SMEM = WARPS * PROF16_BYTES;   // the traceback form with 16-bit lanes
extern __shared__ uint2 g_dyn_prof[];

template <int TIE>
__global__ void __launch_bounds__(WARPS * 32, 2) k_ga(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    void *bnd = (char *)kp.bnd + gw * kp.bnd_bytes;
    uint2 *prof = g_dyn_prof + (threadIdx.x >> 5) * (NCODES * 32);
    unsigned long long exec = 0;
    uint64_t p;
    WarpQueue q;
    uint64_t t;
    while (q.pop(&kp.counter[0], kp.n, t)) {
        p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) { if (lane == 0) atomicOr(kp.status, ST_BAD_SCHED); continue; }
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result best = empty_result();
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            if (lane == 0) { atomicOr(kp.status, ST_BAD_INDEX); kp.out[p] = best; }
            continue;
        }
        uint64_t cells = 0;
        bool have = false, bad = false;
        XdRec r0{0, 0, 0, 0, 0u, XF_NONE};
        for (int s = 0; s < 2; ++s) {
            XdRec rec = kp.xd[2 * p + s];
            if (rec.flags & XF_NONE) continue;
            if (rec.flags & XF_SAME) {
                // the same extension and alignment again
                cells += (uint64_t)r0.cells + (uint64_t)(r0.ev - r0.bv) * (uint64_t)(r0.eh - r0.bh);
                continue;
            }
            if (rec.flags & XF_BAD) bad = true;
            const int bv = rec.bv, ev = rec.ev, bh = rec.bh, eh = rec.eh;
            const uint64_t area = (uint64_t)(ev - bv) * (uint64_t)(eh - bh);
            cells += rec.cells + area;
            const bool same_region = s == 1 && !(r0.flags & XF_NONE) && bv == r0.bv &&
                                     ev == r0.ev && bh == r0.bh && eh == r0.eh;
            if (s == 0) r0 = rec;
            if (same_region) continue;  // identical alignment, cannot win
            const int rm = ev - bv, rn = eh - bh;
            int score;
            uint32_t M, D, G;
            if (rm <= S1::MAXSIDE && rn <= S1::MAXSIDE) {
                const DpOut<S1> d = dp_dispatch<S1, TIE>(V + bv, rm, Hs + bh, rn, ssm, prof, kp.go, kp.ge, bnd, kp.rows_cap);
                score = d.score; M = d.st.M(); D = d.st.D(); G = d.st.G();
            } else {
                const DpOut<S2> d = dp_dispatch<S2, TIE>(V + bv, rm, Hs + bh, rn, ssm, prof, kp.go, kp.ge, bnd, kp.rows_cap);
                score = d.score; M = d.st.M(); D = d.st.D(); G = d.st.G();
            }
            exec += area;
            const uint32_t L = (uint32_t)(rm + rn) - D;
            pg_result cur;
            cur.score = score; cur.aln_len = L; cur.matches = M; cur.gap_opens = G;
            cur.beg_v = (uint16_t)bv; cur.end_v = (uint16_t)ev;
            cur.beg_h = (uint16_t)bh; cur.end_h = (uint16_t)eh;
            cur.seed_used = (uint8_t)s; cur.pad = 0; cur.cells = 0; cur.score_aln = 0.0f;
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
        if (bad) best.flags |= PG_RF_BAD_SEED;
        apply_filter(best, m, n, kp.cov_thr, kp.ani_thr);
        if (lane == 0) kp.out[p] = best;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

// ------------------------------------------------------------------ k_sw
template <int TIE>
__global__ void __launch_bounds__(WARPS * 32) k_sw(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    void *bnd = (char *)kp.bnd + gw * kp.bnd_bytes;
    uint2 *prof = g_dyn_prof + (threadIdx.x >> 5) * (NCODES * 32);
    unsigned long long exec = 0;
    uint64_t p;
    WarpQueue q;
    uint64_t t;
    while (q.pop(&kp.counter[0], kp.n, t)) {
        p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) { if (lane == 0) atomicOr(kp.status, ST_BAD_SCHED); continue; }
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result o = empty_result();
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            if (lane == 0) { atomicOr(kp.status, ST_BAD_INDEX); kp.out[p] = o; }
            continue;
        }
        exec += (unsigned long long)m * (unsigned long long)n;
        o.cells = sat_u32((uint64_t)m * (uint64_t)n);
        int score = 0, have = 0, ei = 0, ej = 0, i0 = 0, j0 = 0;
        uint32_t M = 0, D = 0, G = 0;
        if (m <= L1::MAXSIDE && n <= L1::MAXSIDE) {
            const DpOut<L1> d = dp_dispatch<L1, TIE>(V, m, Hs, n, ssm, prof, kp.go, kp.ge, bnd, kp.rows_cap);
            score = d.score; have = d.have; ei = d.ei; ej = d.ej;
            M = d.st.M(); D = d.st.D(); G = d.st.G(); i0 = d.st.i0(); j0 = d.st.j0();
        } else {
            const DpOut<L2> d = dp_dispatch<L2, TIE>(V, m, Hs, n, ssm, prof, kp.go, kp.ge, bnd, kp.rows_cap);
            score = d.score; have = d.have; ei = d.ei; ej = d.ej;
            M = d.st.M(); D = d.st.D(); G = d.st.G(); i0 = d.st.i0(); j0 = d.st.j0();
        }
        if (have) {
            const uint32_t L = (uint32_t)((ei - i0) + (ej - j0)) - D;
            o.score = score;
            o.aln_len = L; o.matches = M; o.gap_opens = G;
            o.beg_v = (uint16_t)i0; o.end_v = (uint16_t)ei;
            o.beg_h = (uint16_t)j0; o.end_h = (uint16_t)ej;
            if (L > 0) { o.identity = identity_of(M, L); o.flags = 0; }
        }
        apply_filter(o, m, n, kp.cov_thr, kp.ani_thr);
        if (lane == 0) kp.out[p] = o;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

}  // namespace pg
