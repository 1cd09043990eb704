// pg_kernels_dir.cuh -- the traceback form of the alignment kernels (tuning
// option dp_traceback): k_ga_dir / k_sw_dir run dp_warp_dir, or dp_warp_dir16
// on 16-bit lanes for the regions that fit them (dp_traceback 2; one warp per
// region, direction nibbles into an HBM arena); with dp_traceback 3 the 16-bit
// regions of up to 256 rows run two per warp in dp_pair_dir16 (X-drop: in
// k_ga_pair, SW: inside k_sw_dir).  k_tb_ga / k_tb_sw trace them back (one
// thread per pair, pg_trace.cuh) and write the same pg_result records k_ga /
// k_sw write.  A batch whose direction matrices exceed the arena runs in
// chunks of consecutive tasks (bucket order), each chunk DP then traceback.
#pragma once
#include <cstdint>

#include "pg_dpdir.cuh"
#include "pg_dpdir16.cuh"
#include "pg_kernels.cuh"
#include "pg_trace.cuh"

namespace pg {

// rows per lane of the traceback DP: no statistics registers, so up to 8
__device__ __forceinline__ int dir_rows(int m, int cap) { return dp_rows_per_lane<S1>(m, cap); }

// which seeds of an X-drop pair get a DP of their own, with their regions
// (the choices of k_ga: not tried, same seed, same region, empty region)
struct SeedPlan {
    XdRec rec[2];
    bool dp[2];
};

__device__ __forceinline__ SeedPlan seed_plan(const KParams &kp, uint64_t p)
{
    SeedPlan sp;
    sp.rec[0] = kp.xd[2 * p];
    sp.rec[1] = kp.xd[2 * p + 1];
    const XdRec &a = sp.rec[0], &b = sp.rec[1];
    sp.dp[0] = !(a.flags & (XF_NONE | XF_BADIDX)) && a.ev > a.bv && a.eh > a.bh;
    const bool same_region = !(a.flags & XF_NONE) && b.bv == a.bv && b.ev == a.ev &&
                             b.bh == a.bh && b.eh == a.eh;
    sp.dp[1] = !(b.flags & (XF_NONE | XF_SAME | XF_BADIDX)) && !same_region && b.ev > b.bv &&
               b.eh > b.bh;
    return sp;
}

// direction bytes of an m x n region: 16-bit lanes where they run, 32-bit
// otherwise, room for either where a checked region may be redone
__device__ __forceinline__ uint64_t region_bytes(const KParams &kp, int m, int n)
{
    if (dir16_paired(kp, m, n)) return dir16_pair_bytes(m, n);
    const int mode = dir16_mode(kp, m, n);
    const uint64_t b16 = mode ? dir16_bytes(m, n, dir16_rows(m, kp.rows_cap)) : 0;
    const uint64_t b32 = mode != 1 ? dir_bytes(m, n, dir_rows(m, kp.rows_cap)) : 0;
    return b16 > b32 ? b16 : b32;
}

// a region's DP ran on 16-bit lanes (mode, and for a checked region the
// redo flag its DP recorded)
__device__ __forceinline__ bool region16(const KParams &kp, int m, int n, int redone)
{
    const int mode = dir16_mode(kp, m, n);
    return mode == 1 || (mode == 2 && !redone);
}

// rows per lane and lanes of the wavefront of a region's direction words
__device__ __forceinline__ void region_layout(const KParams &kp, int m, int n, bool w16, int &R, int &vl)
{
    if (!w16) { R = dir_rows(m, kp.rows_cap); vl = 32; }
    else if (dir16_paired(kp, m, n)) { R = dir16_pair_rows(m); vl = 32; }
    else { R = dir16_rows(m, kp.rows_cap); vl = 64; }
}

// this warp's score profile in the dynamic shared memory of the traceback DP
__device__ __forceinline__ uint2 *dir_prof(const KParams &kp)
{
    const int per_warp = (kp.dir16_lim > 0 ? PROF16_BYTES : PROF_BYTES) / 8;
    return g_dyn_prof + (threadIdx.x >> 5) * per_warp;
}

// direction bytes of each task (bucket position t)
// direction bytes of each task (bucket position t); *nchk += the checked
// regions (mode 2) among them
template <bool XDROP>
__global__ void k_dirsize(const KParams kp, uint64_t *bytes, unsigned long long *nchk)
{
    unsigned long long chk = 0;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= kp.n;
         t += (uint64_t)gridDim.x * blockDim.x) {
        if (t == kp.n) { bytes[t] = 0; continue; }
        const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
        uint64_t b = 0;
        if (p < kp.n) {
            if (XDROP) {
                const SeedPlan sp = seed_plan(kp, p);
#pragma unroll
                for (int s = 0; s < 2; ++s) {
                    if (!sp.dp[s]) continue;
                    const int rm = sp.rec[s].ev - sp.rec[s].bv, rn = sp.rec[s].eh - sp.rec[s].bh;
                    b += region_bytes(kp, rm, rn);
                    chk += dir16_mode(kp, rm, rn) == 2;
                }
            } else {
                const pg_pair pr = kp.pairs[p];
                const uint8_t *V, *Hs;
                int m, n;
                if (pair_seqs(kp, pr, V, m, Hs, n)) {
                    b = region_bytes(kp, m, n);
                    chk += dir16_mode(kp, m, n) == 2;
                }
            }
        }
        bytes[t] = b;
    }
    if (chk) atomicAdd(nchk, chk);
}

// end of the chunk that starts at task t0: the largest t1 <= n with
// doff[t1] - doff[t0] <= budget, at least t0 + 1
static __global__ void k_chunk_end(const uint64_t *doff, uint64_t t0, uint64_t n, uint64_t budget,
                            uint64_t *t1)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint64_t base = doff[t0];
    uint64_t lo = t0 + 1, hi = n;   // answer in [lo, hi]
    if (doff[lo] - base > budget) { *t1 = lo; return; }
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (doff[mid] - base <= budget) lo = mid; else hi = mid - 1;
    }
    *t1 = lo;
}

// The DP of one region.  CHK false: a region on 16-bit lanes with every value
// provably in range (mode 1) or on 32-bit lanes (mode 0); CHK true: a checked
// region (mode 2), the checked 16-bit form and, if a value left the range, the
// 32-bit form after it (sat = 1: the traceback walks the 32-bit layout).  The
// kernels take checked regions in a pass of their own, so the common pass's
// code stays free of the checked form.
template <int TIE, bool LOCAL, bool CHK>
__device__ __forceinline__ DirOut dp_dispatch_dir(const KParams &kp, const uint8_t *V, int m,
                                                  const uint8_t *Hs, int n, const int *ssm,
                                                  uint2 *prof, void *bnd, uint32_t *dir)
{
    EdgeD *b = (EdgeD *)bnd;
    const int go = kp.go, ge = kp.ge, cap = kp.rows_cap;
    DirOut d;
    if (CHK || dir16_mode(kp, m, n) == 1) {
        switch (dir16_rows(m, cap)) {
        case 1: d = dp_warp_dir16<TIE, 1, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 2: d = dp_warp_dir16<TIE, 2, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 3: d = dp_warp_dir16<TIE, 3, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 4: d = dp_warp_dir16<TIE, 4, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 5: d = dp_warp_dir16<TIE, 5, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 6: d = dp_warp_dir16<TIE, 6, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        case 7: d = dp_warp_dir16<TIE, 7, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        default: d = dp_warp_dir16<TIE, 8, LOCAL, CHK>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
        }
        if (!CHK || !d.sat) return d;
        // a value left int16's safe range: redo the region on 32-bit lanes (the
        // profile buffer and arena slot hold either form)
    }
    switch (dir_rows(m, cap)) {
    case 1: d = dp_warp_dir<TIE, 1, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 2: d = dp_warp_dir<TIE, 2, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 3: d = dp_warp_dir<TIE, 3, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 4: d = dp_warp_dir<TIE, 4, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 5: d = dp_warp_dir<TIE, 5, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 6: d = dp_warp_dir<TIE, 6, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    case 7: d = dp_warp_dir<TIE, 7, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    default: d = dp_warp_dir<TIE, 8, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, b, dir); break;
    }
    d.sat = CHK ? 1 : 0;
    return d;
}

// the DP of two regions of R rows per lane on the two halves of the warp (each
// lane passes its own half's region; m = 0: none)
template <int TIE, bool LOCAL>
__device__ __forceinline__ DirOut dp_dispatch_pair(const KParams &kp, int R, const uint8_t *V, int m,
                                                   const uint8_t *Hs, int n, const int *ssm,
                                                   uint2 *prof, uint32_t *dir)
{
    const int go = kp.go, ge = kp.ge;
    switch (R) {
    case 1: return dp_pair_dir16<TIE, 1, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 2: return dp_pair_dir16<TIE, 2, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 3: return dp_pair_dir16<TIE, 3, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 4: return dp_pair_dir16<TIE, 4, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 5: return dp_pair_dir16<TIE, 5, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 6: return dp_pair_dir16<TIE, 6, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    case 7: return dp_pair_dir16<TIE, 7, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    default: return dp_pair_dir16<TIE, 8, LOCAL>(V, m, Hs, n, ssm, prof, go, ge, dir);
    }
}

// A region waiting for a partner of the same rows per lane: lane R of the warp
// holds key + 1 of the waiting region of R rows per lane (0: none).  X-drop key:
// task << 1 | seed; SW key: task.
struct PairSlots {
    uint64_t pend = 0;
    // the waiting key + 1 for R (0: none); the slot is then empty, or holds key + 1
    __device__ __forceinline__ uint64_t swap(int R, uint64_t key1)
    {
        const int lane = threadIdx.x & 31;
        const uint64_t w = __shfl_sync(FULL, pend, R);
        if (lane == R) pend = w ? 0 : key1;
        return w;
    }
};

// seed s's region of the X-drop task at bucket position t: sequences, sides
// and arena offset (from the chunk's base); false when the pair has no such DP
__device__ __forceinline__ bool ga_region(const KParams &kp, uint64_t t, int s, const uint64_t *doff,
                                          uint64_t base, uint64_t &p, const uint8_t *&V, int &m,
                                          const uint8_t *&Hs, int &n, uint64_t &off)
{
    p = kp.order ? (uint64_t)kp.order[t] : t;
    if (p >= kp.n) return false;
    const pg_pair pr = kp.pairs[p];
    int pm, pn;
    if (!pair_seqs(kp, pr, V, pm, Hs, pn)) return false;
    const SeedPlan sp = seed_plan(kp, p);
    if (!sp.dp[s]) return false;
    off = doff[t] - base;
    if (s == 1 && sp.dp[0])
        off += region_bytes(kp, sp.rec[0].ev - sp.rec[0].bv, sp.rec[0].eh - sp.rec[0].bh);
    const XdRec r = s ? sp.rec[1] : sp.rec[0];
    V += r.bv; Hs += r.bh;
    m = r.ev - r.bv; n = r.eh - r.bh;
    return true;
}

// the DP of two waiting X-drop regions (keys a and b, + 1; b = 0: none)
template <int TIE>
__device__ __forceinline__ void ga_pair(const KParams &kp, int R, uint64_t a1, uint64_t b1, uint64_t t0,
                                        const uint64_t *doff, uint64_t base, uint8_t *arena,
                                        const int *ssm, uint2 *prof, int *dsc)
{
    const int lane = threadIdx.x & 31;
    const uint64_t k1 = lane < 16 ? a1 : b1;
    uint64_t p = 0, off = 0;
    const uint8_t *V = nullptr, *Hs = nullptr;
    int m = 0, n = 0;
    const int s = k1 ? (int)((k1 - 1) & 1) : 0;
    if (!k1 || !ga_region(kp, t0 + ((k1 - 1) >> 1), s, doff, base, p, V, m, Hs, n, off)) m = n = 0;
    const DirOut d = dp_dispatch_pair<TIE, false>(kp, R, V, m, Hs, n, ssm, prof, (uint32_t *)(arena + off));
    if ((lane & 15) == 0 && m > 0) { dsc[2 * p + s] = d.score; dsc[2 * kp.n + 2 * p + s] = 0; }
}

// ---------------------------------------------------------------- X-drop
// DP of each seed region of the tasks [t0, t1); a task's regions sit at
// arena + doff[t] - doff[t0] (seed 0 first).  dsc[2p + s] = global score,
// dsc[2n + 2p + s] = 1 where a checked 16-bit region was redone on 32-bit lanes.
template <int TIE, bool CHK>
__global__ void __launch_bounds__(WARPS * 32, 2) k_ga_dir(const KParams kp, uint64_t t0, uint64_t t1,
                                                         const uint64_t *doff, uint8_t *arena, int *dsc)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    void *bnd = (char *)kp.bnd + gw * kp.bnd_bytes;
    uint2 *prof = dir_prof(kp);
    const int lane = threadIdx.x & 31;
    unsigned long long exec = 0;
    const uint64_t base = doff[t0];
    WarpQueue q;
    uint64_t u;
    while (q.pop(&kp.counter[CHK ? 0 : 3], t1 - t0, u)) {
        const uint64_t t = t0 + u;
        const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) continue;
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        if (!pair_seqs(kp, pr, V, m, Hs, n)) continue;
        const SeedPlan sp = seed_plan(kp, p);
        uint64_t off = doff[t] - base;
        // one copy of the DP dispatch for both seeds (its instantiations are many)
#pragma unroll 1
        for (int s = 0; s < 2; ++s) {
            if (!sp.dp[s]) continue;
            const XdRec &r = sp.rec[s];
            const int rm = r.ev - r.bv, rn = r.eh - r.bh;
            // this pass's regions only (the half-warp ones run in k_ga_pair)
            if ((dir16_mode(kp, rm, rn) == 2) == CHK && (CHK || !dir16_paired(kp, rm, rn))) {
                const DirOut d = dp_dispatch_dir<TIE, false, CHK>(kp, V + r.bv, rm, Hs + r.bh, rn, ssm,
                                                                  prof, bnd, (uint32_t *)(arena + off));
                if (lane == 0) { dsc[2 * p + s] = d.score; dsc[2 * kp.n + 2 * p + s] = d.sat; }
                exec += (uint64_t)rm * (uint64_t)rn;
            }
            off += region_bytes(kp, rm, rn);
        }
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

// DP of the half-warp regions (dir16_paired) of the tasks [t0, t1), two per
// warp: a region waits for a partner of the same rows per lane, and those left
// without one when the queue runs dry run alone.  A kernel of its own: with
// both in k_ga_dir, its whole-warp regions ran 26 % slower.
template <int TIE>
__global__ void __launch_bounds__(WARPS * 32, 2) k_ga_pair(const KParams kp, uint64_t t0, uint64_t t1,
                                                          const uint64_t *doff, uint8_t *arena, int *dsc)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    uint2 *prof = dir_prof(kp);
    const int lane = threadIdx.x & 31;
    unsigned long long exec = 0;
    const uint64_t base = doff[t0];
    WarpQueue q;
    PairSlots slots;
    // one call site of the DP (its instantiations are many): each turn finds
    // the next two regions, seed by seed, then (flush = R, 1..8) the ones left
    uint64_t u = 0;
    int s = 2, flush = 0;           // next seed of the task (2: take a task)
    SeedPlan sp;
    for (;;) {
        uint64_t a1 = 0, b1 = 0;
        int R = 0;
        if (flush == 0) {
            if (s == 2) {
                if (!q.pop(&kp.counter[0], t1 - t0, u)) { flush = 1; continue; }
                const uint64_t t = t0 + u;
                const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
                if (p >= kp.n) continue;
                sp = seed_plan(kp, p);
                s = 0;
            }
            const int js = s++;
            if (!sp.dp[js]) continue;
            const XdRec r = js ? sp.rec[1] : sp.rec[0];
            const int rm = r.ev - r.bv, rn = r.eh - r.bh;
            if (!dir16_paired(kp, rm, rn)) continue;
            exec += (uint64_t)rm * (uint64_t)rn;
            R = dir16_pair_rows(rm);
            b1 = ((u << 1) | (uint64_t)js) + 1;
            a1 = slots.swap(R, b1);
            if (!a1) continue;
        } else {
            if (flush > 8) break;
            R = flush++;
            a1 = __shfl_sync(FULL, slots.pend, R);
            if (!a1) continue;
        }
        ga_pair<TIE>(kp, R, a1, b1, t0, doff, base, arena, ssm, prof, dsc);
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

// both seeds' walks of one pair, stepped together (two independent chains of
// direction loads in flight per thread)
template <bool WA, bool WB>
__device__ __forceinline__ void walk_both(const KParams &kp, const uint32_t *const dm[2], const int rm[2],
                                          const int rn[2], const uint8_t *const V[2],
                                          const uint8_t *const Hs[2], const int *ssm,
                                          const bool act[2], TraceOut tr[2])
{
    int Ra, vla, Rb, vlb;
    region_layout(kp, rm[0], rn[0], WA, Ra, vla);
    region_layout(kp, rm[1], rn[1], WB, Rb, vlb);
    Walker<false, WA> a(dm[0], rn[0], Ra, vla, rm[0], rn[0], V[0], Hs[0], ssm, kp.go, kp.ge, 0);
    Walker<false, WB> b(dm[1], rn[1], Rb, vlb, rm[1], rn[1], V[1], Hs[1], ssm, kp.go, kp.ge, 0);
    a.done = !act[0];
    b.done = !act[1];
    while (a.step() | b.step()) {}
    tr[0] = a.out();
    tr[1] = b.out();
}

// traceback and result of the tasks [t0, t1), one thread per task: the same
// record k_ga writes.  Five resident blocks per SM (48 registers, a few
// spilled) measured 1 % faster than four: the walks wait on memory, so more
// of them in flight count for more than the spills.
static __global__ void __launch_bounds__(256, 5) k_tb_ga(const KParams kp, uint64_t t0, uint64_t t1,
                                               const uint64_t *doff, const uint8_t *arena,
                                               const int *dsc)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const uint64_t base = doff[t0];
    const int gmax = kp.go > kp.ge ? kp.go : kp.ge;
    for (uint64_t t = t0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < t1;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) { atomicOr(kp.status, ST_BAD_SCHED); continue; }
        const pg_pair pr = kp.pairs[p];
        const uint8_t *Vs, *Hss;
        int m, n;
        pg_result best = empty_result();
        if (!pair_seqs(kp, pr, Vs, m, Hss, n)) {
            atomicOr(kp.status, ST_BAD_INDEX);
            kp.out[p] = best;
            continue;
        }
        const SeedPlan sp = seed_plan(kp, p);
        // each seed's region, and which of them have a DP to walk back
        uint64_t off = doff[t] - base;
        uint64_t cells = 0;
        bool bad = false, use[2], act[2], w16[2];
        const uint32_t *dm[2];
        const uint8_t *V[2], *Hs[2];
        int rm[2], rn[2];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const XdRec &rec = sp.rec[s];
            use[s] = act[s] = w16[s] = false;
            rm[s] = rn[s] = 0;
            dm[s] = nullptr; V[s] = Vs; Hs[s] = Hss;
            if (rec.flags & XF_NONE) continue;
            if (rec.flags & XF_SAME) {
                const XdRec &r0 = sp.rec[0];
                cells += (uint64_t)r0.cells + (uint64_t)(r0.ev - r0.bv) * (uint64_t)(r0.eh - r0.bh);
                continue;
            }
            if (rec.flags & XF_BAD) bad = true;
            rm[s] = rec.ev - rec.bv;
            rn[s] = rec.eh - rec.bh;
            cells += rec.cells + (uint64_t)rm[s] * (uint64_t)rn[s];
            const bool same_region = s == 1 && !(sp.rec[0].flags & XF_NONE) && rec.bv == sp.rec[0].bv &&
                                     rec.ev == sp.rec[0].ev && rec.bh == sp.rec[0].bh && rec.eh == sp.rec[0].eh;
            if (same_region) continue;
            use[s] = true;
            V[s] = Vs + rec.bv;
            Hs[s] = Hss + rec.bh;
            if (rm[s] > 0 && rn[s] > 0) {
                act[s] = true;
                w16[s] = region16(kp, rm[s], rn[s], dsc[2 * kp.n + 2 * p + s]);
                dm[s] = (const uint32_t *)(arena + off);
                off += region_bytes(kp, rm[s], rn[s]);
            }
        }
        TraceOut tr[2];
        if (w16[0] && w16[1]) walk_both<true, true>(kp, dm, rm, rn, V, Hs, ssm, act, tr);
        else if (w16[0]) walk_both<true, false>(kp, dm, rm, rn, V, Hs, ssm, act, tr);
        else if (w16[1]) walk_both<false, true>(kp, dm, rm, rn, V, Hs, ssm, act, tr);
        else walk_both<false, false>(kp, dm, rm, rn, V, Hs, ssm, act, tr);
        bool have = false;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!use[s]) continue;
            const XdRec &rec = sp.rec[s];
            int score;
            uint32_t M = 0, D = 0, G = 0;
            if (act[s]) {
                score = dsc[2 * p + s];
                M = tr[s].M; D = tr[s].D; G = tr[s].G;
            } else if (rm[s] + rn[s] > 0) {
                score = kp.go + (rm[s] + rn[s] - 1) * gmax;   // one gap run
                G = 1;
            } else {
                score = 0;
            }
            const uint32_t L = (uint32_t)(rm[s] + rn[s]) - D;
            pg_result cur;
            cur.score = score; cur.aln_len = L; cur.matches = M; cur.gap_opens = G;
            cur.beg_v = rec.bv; cur.end_v = rec.ev;
            cur.beg_h = rec.bh; cur.end_h = rec.eh;
            cur.seed_used = (uint8_t)s; cur.pad = 0; cur.cells = 0; cur.score_aln = 0.0f;
            if (L == 0) { cur.identity = 0.0f; cur.flags = PG_RF_EMPTY; }
            else { cur.identity = identity_of(M, L); cur.flags = 0; }
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
        kp.out[p] = best;
    }
}

// ---------------------------------------------------------------- SW
// the DP of two waiting SW pairs (task keys a and b, + 1; b = 0: none)
template <int TIE>
__device__ __forceinline__ void sw_pair(const KParams &kp, int R, uint64_t a1, uint64_t b1, uint64_t t0,
                                        const uint64_t *doff, uint64_t base, uint8_t *arena,
                                        const int *ssm, uint2 *prof, int *dsc)
{
    const int lane = threadIdx.x & 31;
    const uint64_t k1 = lane < 16 ? a1 : b1;
    uint64_t p = 0, off = 0;
    const uint8_t *V = nullptr, *Hs = nullptr;
    int m = 0, n = 0;
    if (k1) {
        const uint64_t t = t0 + (k1 - 1);
        p = kp.order ? (uint64_t)kp.order[t] : t;
        const pg_pair pr = kp.pairs[p];
        if (!pair_seqs(kp, pr, V, m, Hs, n)) m = n = 0;
        off = doff[t] - base;
    }
    const DirOut d = dp_dispatch_pair<TIE, true>(kp, R, V, m, Hs, n, ssm, prof, (uint32_t *)(arena + off));
    if ((lane & 15) == 0 && m > 0) {
        int4 *o = reinterpret_cast<int4 *>(dsc) + p;
        *o = make_int4(d.score, d.ei, d.ej, d.have);
    }
}

// local DP of the tasks [t0, t1); dsc[4p ..] = score, end row, end column,
// have | 2 if a checked 16-bit region was redone on 32-bit lanes.  The
// half-warp pairs (dir16_paired) run here too, two per warp: a pair waits for
// a partner of the same rows per lane, and those left without one run alone
// at the end.  (A pass of their own, as X-drop's k_ga_pair, measured 5 %
// slower here: sw100k is 10 ms, and a second pass adds a second tail.)
template <int TIE, bool CHK>
__global__ void __launch_bounds__(WARPS * 32, 2) k_sw_dir(const KParams kp, uint64_t t0, uint64_t t1,
                                                      const uint64_t *doff, uint8_t *arena, int *dsc)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    void *bnd = (char *)kp.bnd + gw * kp.bnd_bytes;
    uint2 *prof = dir_prof(kp);
    const int lane = threadIdx.x & 31;
    unsigned long long exec = 0;
    const uint64_t base = doff[t0];
    WarpQueue q;
    PairSlots slots;
    uint64_t u;
    while (q.pop(&kp.counter[CHK ? 0 : 3], t1 - t0, u)) {
        const uint64_t t = t0 + u;
        const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) continue;
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        if (!pair_seqs(kp, pr, V, m, Hs, n)) continue;
        if ((dir16_mode(kp, m, n) == 2) != CHK) continue;   // this pass's pairs only
        exec += (unsigned long long)m * (unsigned long long)n;
        if (!CHK && dir16_paired(kp, m, n)) {
            // half a warp: wait for a partner of the same rows per lane
            const int R = dir16_pair_rows(m);
            const uint64_t w1 = slots.swap(R, u + 1);
            if (w1) sw_pair<TIE>(kp, R, w1, u + 1, t0, doff, base, arena, ssm, prof, dsc);
            continue;
        }
        DirOut d;
        d.score = 0; d.ei = 0; d.ej = 0; d.have = 0;
        if (m > 0 && n > 0)
            d = dp_dispatch_dir<TIE, true, CHK>(kp, V, m, Hs, n, ssm, prof, bnd,
                                                (uint32_t *)(arena + (doff[t] - base)));
        if (lane == 0) {
            int4 *o = reinterpret_cast<int4 *>(dsc) + p;
            *o = make_int4(d.score, d.ei, d.ej, d.have | (d.sat << 1));
        }
    }
    if (!CHK && kp.dir16_pair) {
        // pairs left without a partner run on half a warp alone
#pragma unroll 1
        for (int R = 1; R <= 8; ++R) {
            const uint64_t w1 = __shfl_sync(FULL, slots.pend, R);
            if (w1) sw_pair<TIE>(kp, R, w1, 0, t0, doff, base, arena, ssm, prof, dsc);
        }
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

// traceback and result of the tasks [t0, t1), one thread per task: the same
// record k_sw writes
static __global__ void __launch_bounds__(256) k_tb_sw(const KParams kp, uint64_t t0, uint64_t t1,
                                               const uint64_t *doff, const uint8_t *arena,
                                               const int *dsc)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const uint64_t base = doff[t0];
    for (uint64_t t = t0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < t1;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = kp.order ? (uint64_t)kp.order[t] : t;
        if (p >= kp.n) { atomicOr(kp.status, ST_BAD_SCHED); continue; }
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result o = empty_result();
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            atomicOr(kp.status, ST_BAD_INDEX);
            kp.out[p] = o;
            continue;
        }
        o.cells = sat_u32((uint64_t)m * (uint64_t)n);
        const int4 d = reinterpret_cast<const int4 *>(dsc)[p];
        if (m > 0 && n > 0 && (d.w & 1)) {
            const uint32_t *dm = (const uint32_t *)(arena + (doff[t] - base));
            const bool w16 = region16(kp, m, n, d.w >> 1);
            int R, vl;
            region_layout(kp, m, n, w16, R, vl);
            const TraceOut tr = w16 ? trace_walk<true, true>(dm, n, R, vl, d.y, d.z, V, Hs, ssm, kp.go, kp.ge, d.x)
                                    : trace_walk<true, false>(dm, n, R, vl, d.y, d.z, V, Hs, ssm, kp.go, kp.ge, d.x);
            const uint32_t L = (uint32_t)((d.y - tr.i0) + (d.z - tr.j0)) - tr.D;
            o.score = d.x;
            o.aln_len = L; o.matches = tr.M; o.gap_opens = tr.G;
            o.beg_v = (uint16_t)tr.i0; o.end_v = (uint16_t)d.y;
            o.beg_h = (uint16_t)tr.j0; o.end_h = (uint16_t)d.z;
            if (L > 0) { o.identity = identity_of(tr.M, L); o.flags = 0; }
        }
        apply_filter(o, m, n, kp.cov_thr, kp.ani_thr);
        kp.out[p] = o;
    }
}

}  // namespace pg
