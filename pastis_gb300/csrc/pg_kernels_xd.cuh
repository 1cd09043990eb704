// pg_kernels_xd.cuh -- the X-drop extension kernels (one definition: only
// pg_api.cu includes this file): k_xdr, thread per (pair, seed) task with the
// band window in registers (pg_xdreg.cuh), the default; k_xdf and k_xd,
// thread per task with the 32-bit band in a shared-memory ring (pg_xdrop.cuh),
// stepping one direction at a time or running each task to its end (tuning
// option xd_stepped); k_xd16, a thread per task on 16-bit lanes (tuning option
// xd_int16); k_xd_wide, warp per task for the bands that overflow a thread's
// window or ring.
#pragma once
#include <cstdint>

#include "pg_kernels.cuh"
#include "pg_xdreg.cuh"

namespace pg {

// ------------------------------------------------------------------ k_xd
// One thread per (pair, seed) task, run to its end before the thread takes
// the next: fewer registers than k_xdf (7 resident blocks per SM against 5),
// which wins when the residues stream from DRAM (sequence sets larger than
// L2); a warp waits on its longest extension.
__global__ void __launch_bounds__(XT) k_xd(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    __shared__ int ring[3 * XW * XT];
    load_sm(ssm, kp.sm);
    __syncthreads();
    int *base = ring + threadIdx.x;
    const uint64_t ntask = 2 * kp.n;
    unsigned long long exec = 0;
    for (;;) {
        const uint64_t task = atomicAdd(&kp.counter[1], 1u);
        if (task >= ntask) break;
        const uint64_t p = task >> 1;
        const int s = (int)(task & 1);
        const pg_pair pr = kp.pairs[p];
        XdRec rec{0, 0, 0, 0, 0u, 0u};
        const uint8_t *V, *Hs;
        int m, n;
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            rec.flags = XF_BADIDX;
        } else if (s >= kp.seed_count ||
                   (s == 1 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && pr.count < 2)) {
            rec.flags = XF_NONE;
        } else if (s == 1 && pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0) {
            rec.flags = XF_SAME;
        } else {
            int bv, ev, bh, eh;
            if (seed_region(kp, pr, s, m, n, bv, ev, bh, eh)) rec.flags |= XF_BAD;
            bool ok = true;
            if (bv > 0 && bh > 0) {
                const XdOut x = xdrop_dir_thread<XW, XT>(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1,
                                                         ssm, kp.xg, kp.xdrop, base);
                ok = x.ok;
                rec.cells += x.cells;
                bv -= x.dv; bh -= x.dh;
            }
            if (ok && ev < m && eh < n) {
                const XdOut x = xdrop_dir_thread<XW, XT>(V + ev, m - ev, 1, Hs + eh, n - eh, 1,
                                                         ssm, kp.xg, kp.xdrop, base);
                ok = x.ok;
                rec.cells += x.cells;
                ev += x.dv; eh += x.dh;
            }
            if (ok) {
                rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev;
                rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
                exec += rec.cells;
            } else {
                rec.flags |= XF_OVF;
                rec.cells = 0;
                const unsigned int slot = atomicAdd(&kp.counter[2], 1u);
                kp.ovf[slot] = (uint32_t)task;
            }
        }
        kp.xd[task] = rec;
    }
    if (exec) atomicAdd(kp.exec_cells, exec);
}

// ------------------------------------------------------------------ k_xdf
// One thread per (pair, seed) task, each thread stepping one extension
// direction at a time: when a direction ends the thread starts the next one
// at once (the task's other direction, or the next task).  Running each task
// to its end before taking the next, as an earlier kernel did, left a warp
// waiting on its longest extension: 6.5 of 32 lanes active per instruction,
// 28.6 ms per 1M pairs against 16.8 ms here (xdrop1m, sequences in L2).  The next tasks' inputs are read ahead
// in three stages (work counter, pair record, sequence offsets), each
// consumed a task later, so starting a task waits on no memory.  A band
// wider than the 16-slot ring sends the task to the overflow list for
// k_xd_wide.
// a task in the read-ahead pipeline: id, then its pair record, then what
// starting it needs (flags, its seed, its sequences' offsets)
constexpr uint32_t XFT_VALID = 1, XFT_IDX = 2, XFT_SAME = 4, XFT_FEW = 8;
struct XfReady {
    uint32_t t, flags, seed;   // seed: rs | cs << 16 of the task's seed
    uint64_t r0, r1, c0, c1;
};

__global__ void __launch_bounds__(XT) k_xdf(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    __shared__ int ring[3 * XW * XT];
    load_sm(ssm, kp.sm);
    __syncthreads();
    int *base = ring + threadIdx.x;
    const uint32_t ntask = (uint32_t)(2 * kp.n);
    unsigned long long exec = 0;
    // read-ahead pipeline: ta (task id), tb + pb (pair record), c (ready)
    uint32_t ta, tb;
    pg_pair pb;
    XfReady c;
    auto load_pair = [&](uint32_t t, pg_pair &pr) {
        if (t < ntask) pr = kp.pairs[t >> 1];
    };
    auto make_ready = [&](uint32_t t, const pg_pair &pr, XfReady &x) {
        x.t = t;
        x.flags = 0;
        if (t >= ntask) return;
        x.flags = XFT_VALID;
        const uint64_t r = (uint64_t)pr.row + kp.roff, cc = (uint64_t)pr.col + kp.coff;
        const int s = (int)(t & 1);
        x.seed = s ? ((uint32_t)pr.rs1 | ((uint32_t)pr.cs1 << 16)) : ((uint32_t)pr.rs0 | ((uint32_t)pr.cs0 << 16));
        if (pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0) x.flags |= XFT_SAME;
        if (pr.count < 2) x.flags |= XFT_FEW;
        if (r >= kp.nr || cc >= kp.nc) return;
        x.flags |= XFT_IDX;
        x.r0 = kp.roffs[r]; x.r1 = kp.roffs[r + 1];
        x.c0 = kp.coffs[cc]; x.c1 = kp.coffs[cc + 1];
    };
    {
        const uint32_t t0 = atomicAdd(&kp.counter[1], 1u);
        pg_pair p0;
        load_pair(t0, p0);
        make_ready(t0, p0, c);
        tb = atomicAdd(&kp.counter[1], 1u);
        load_pair(tb, pb);
        ta = atomicAdd(&kp.counter[1], 1u);
    }

    XdDir<XW, XT> dir;
    XdRec rec{0, 0, 0, 0, 0u, 0u};
    uint32_t task = 0;
    const uint8_t *V = nullptr, *Hs = nullptr;
    int m = 0, n = 0, bv = 0, ev = 0, bh = 0, eh = 0;
    int phase = 0;     // 0: start a task, 1: left direction running, 2: right direction running
    auto write_rec = [&]() {
        if (rec.flags & XF_OVF) {
            rec.cells = 0;
            const unsigned int slot = atomicAdd(&kp.counter[2], 1u);
            kp.ovf[slot] = task;
        } else if (!(rec.flags & (XF_NONE | XF_SAME | XF_BADIDX))) {
            rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev;
            rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
            exec += rec.cells;
        }
        kp.xd[task] = rec;
    };
    for (;;) {
        while (phase == 0) {
            if (!(c.flags & XFT_VALID)) break;
            // take c, move the pipeline on by one task
            const XfReady cur = c;
            make_ready(tb, pb, c);
            tb = ta;
            load_pair(tb, pb);
            ta = atomicAdd(&kp.counter[1], 1u);
            task = cur.t;
            const int s = (int)(task & 1);
            rec = XdRec{0, 0, 0, 0, 0u, 0u};
            if (!(cur.flags & XFT_IDX)) {
                rec.flags = XF_BADIDX;
            } else if (s >= kp.seed_count ||
                       (s == 1 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && (cur.flags & XFT_FEW))) {
                rec.flags = XF_NONE;
            } else if (s == 1 && (cur.flags & XFT_SAME)) {
                rec.flags = XF_SAME;
            } else {
                V = kp.rseq + cur.r0; m = (int)(cur.r1 - cur.r0);
                Hs = kp.cseq + cur.c0; n = (int)(cur.c1 - cur.c0);
                // seed_region for the task's seed
                bv = (int)(cur.seed & 0xffffu); bh = (int)(cur.seed >> 16);
                ev = bv + kp.seed_len; eh = bh + kp.seed_len;
                if (ev > m || eh > n) {
                    bv = min(bv, m); ev = min(ev, m); bh = min(bh, n); eh = min(eh, n);
                    rec.flags |= XF_BAD;
                }
                if (bv > 0 && bh > 0) {
                    dir.init(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1, kp.xg, kp.xdrop, base);
                    phase = 1;
                } else if (ev < m && eh < n) {
                    dir.init(V + ev, m - ev, 1, Hs + eh, n - eh, 1, kp.xg, kp.xdrop, base);
                    phase = 2;
                }
            }
            if (phase == 0) write_rec();
        }
        if (phase == 0) break;          // no task left for this thread
        if (dir.step(ssm, kp.xg, kp.xdrop, base)) continue;
        const XdOut x = dir.finish(base);
        rec.cells += x.cells;
        if (!x.ok) {
            rec.flags |= XF_OVF;
            write_rec();
            phase = 0;
        } else if (phase == 1) {
            bv -= x.dv; bh -= x.dh;
            if (ev < m && eh < n) {
                dir.init(V + ev, m - ev, 1, Hs + eh, n - eh, 1, kp.xg, kp.xdrop, base);
                phase = 2;
            } else {
                write_rec();
                phase = 0;
            }
        } else {
            ev += x.dv; eh += x.dh;
            write_rec();
            phase = 0;
        }
    }
    if (exec) atomicAdd(kp.exec_cells, exec);
}

// --------------------------------------------------- extension task order
// Threads take extension tasks from a shared counter, so a thread that picks
// up a long task near the end of the batch leaves its warp's other lanes
// idle until it finishes.  Taking the tasks longest first fixes that: their
// length is not known beforehand, but the anti-diagonals a seed's two
// directions can reach are bounded by the residues left of it and right of
// it on both sequences, and ordering by that bound (in quarter octaves)
// gives nearly the ideal finish (a simulation over task lengths of this
// workload: 1.01 of the mean thread load against 1.23 in input order).
// Tasks that run no extension (a second seed equal to the first, or switched
// off) sit in bucket 0, last.
__device__ __forceinline__ int xtask_bucket(const KParams &kp, const pg_pair &pr, int s, int m, int n)
{
    if (s >= kp.seed_count || (s == 1 && pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0)) return 0;
    const int rs = s ? pr.rs1 : pr.rs0, cs = s ? pr.cs1 : pr.cs0;
    const int left = max(0, min(min(rs, cs), min(m, n)));
    const int right = max(0, min(m - rs - kp.seed_len, n - cs - kp.seed_len));
    const uint32_t b = (uint32_t)(left + right) + 2u;    // >= 2
    const int e = 31 - __clz(b);
    const int q = 4 * e + (int)((b << 2 >> e) & 3u);
    return min(XBUCKET - 1, q);
}

// the two tasks of pair p and their buckets (both 0 when the pair's indices
// are out of range: the extension kernel reports those itself)
__device__ __forceinline__ void xtask_buckets(const KParams &kp, uint64_t p, int &b0, int &b1)
{
    const pg_pair pr = kp.pairs[p];
    const uint64_t r = (uint64_t)pr.row + kp.roff, c = (uint64_t)pr.col + kp.coff;
    b0 = b1 = 0;
    if (r >= kp.nr || c >= kp.nc) return;
    const int m = (int)(kp.roffs[r + 1] - kp.roffs[r]), n = (int)(kp.coffs[c + 1] - kp.coffs[c]);
    b0 = xtask_bucket(kp, pr, 0, m, n);
    b1 = xtask_bucket(kp, pr, 1, m, n);
}

__global__ void __launch_bounds__(256) k_xtask_hist(const KParams kp)
{
    __shared__ unsigned int h[XBUCKET];
    for (int b = threadIdx.x; b < XBUCKET; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < kp.n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        int b0, b1;
        xtask_buckets(kp, p, b0, b1);
        atomicAdd(&h[b0], 1u);
        atomicAdd(&h[b1], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < XBUCKET; b += blockDim.x)
        if (h[b]) atomicAdd(&kp.xsched[b], h[b]);
}

// xorder[]: task ids, highest bucket first (any order inside a bucket)
__global__ void __launch_bounds__(256) k_xtask_bucket(const KParams kp)
{
    __shared__ unsigned int start[XBUCKET], h[XBUCKET], base[XBUCKET];
    if (threadIdx.x == 0) {
        unsigned int acc = 0;
        for (int b = XBUCKET - 1; b >= 0; --b) { start[b] = acc; acc += kp.xsched[b]; }
    }
    uint32_t *order = const_cast<uint32_t *>(kp.xorder);
    const uint64_t ntask = 2 * kp.n;
    for (uint64_t c0 = (uint64_t)blockIdx.x * blockDim.x; c0 < kp.n; c0 += (uint64_t)gridDim.x * blockDim.x) {
        for (int b = threadIdx.x; b < XBUCKET; b += blockDim.x) h[b] = 0;
        __syncthreads();
        const uint64_t p = c0 + threadIdx.x;
        int b0 = 0, b1 = 0;
        unsigned int r0 = 0, r1 = 0;
        if (p < kp.n) {
            xtask_buckets(kp, p, b0, b1);
            r0 = atomicAdd(&h[b0], 1u);
            r1 = atomicAdd(&h[b1], 1u);
        }
        __syncthreads();
        for (int b = threadIdx.x; b < XBUCKET; b += blockDim.x)
            if (h[b]) base[b] = start[b] + atomicAdd(&kp.xsched[XBUCKET + b], h[b]);
        __syncthreads();
        if (p < kp.n) {
            const uint64_t q0 = (uint64_t)base[b0] + r0, q1 = (uint64_t)base[b1] + r1;
            if (q0 < ntask && q1 < ntask) {
                order[q0] = (uint32_t)(2 * p);
                order[q1] = (uint32_t)(2 * p + 1);
            } else {
                atomicOr(kp.status, ST_BAD_SCHED);
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ k_xdr
// One thread per (pair, seed) task with the band window in registers
// (XrDirT<NW>): every step computes the 2 NW window columns with packed 16-bit
// operations and no branch on the band, so a warp's threads step together
// whatever their band widths.  Tasks are taken (longest length bound first
// when kp.xorder is set) and their inputs read ahead as in k_xdf; a direction
// starts the moment the previous one ends.  A window wider than 2 NW - 1
// columns sends the task to the overflow list for k_xd_wide.  NW = 8 runs:
// a 12-slot window (NW = 6) executed 15 % fewer instructions on xdrop1m, but
// the 4 % of tasks that outgrew it, rerun on 16 slots in a launch of their
// own, were long homolog extensions at a tenth of the warps, and the
// extension took 9.85 ms per 1M pairs against 9.3.
// Needs xdr_supported(xg, xdrop).
template <int NW>
__global__ void __launch_bounds__(XT) k_xdr(const KParams kp)
{
    __shared__ int ssm[PG_NRES * XR_STRIDE];
    load_sm33(ssm, kp.sm);
    __syncthreads();
    const char *tbl = reinterpret_cast<const char *>(ssm);
    const uint32_t ntask = (uint32_t)(2 * kp.n);
    unsigned long long exec = 0;
    uint32_t ta, tb;
    pg_pair pb;
    XfReady c;
    // the next task: through the longest-first order when there is one
    auto fetch = [&]() -> uint32_t {
        const uint32_t i = atomicAdd(&kp.counter[1], 1u);
        return (kp.xorder && i < ntask) ? kp.xorder[i] : i;
    };
    auto load_pair = [&](uint32_t t, pg_pair &pr) {
        if (t < ntask) pr = kp.pairs[t >> 1];
    };
    auto make_ready = [&](uint32_t t, const pg_pair &pr, XfReady &x) {
        x.t = t;
        x.flags = 0;
        if (t >= ntask) return;
        x.flags = XFT_VALID;
        const uint64_t r = (uint64_t)pr.row + kp.roff, cc = (uint64_t)pr.col + kp.coff;
        const int s = (int)(t & 1);
        x.seed = s ? ((uint32_t)pr.rs1 | ((uint32_t)pr.cs1 << 16)) : ((uint32_t)pr.rs0 | ((uint32_t)pr.cs0 << 16));
        if (pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0) x.flags |= XFT_SAME;
        if (pr.count < 2) x.flags |= XFT_FEW;
        if (r >= kp.nr || cc >= kp.nc) return;
        x.flags |= XFT_IDX;
        x.r0 = kp.roffs[r]; x.r1 = kp.roffs[r + 1];
        x.c0 = kp.coffs[cc]; x.c1 = kp.coffs[cc + 1];
    };
    {
        const uint32_t t0 = fetch();
        pg_pair p0;
        load_pair(t0, p0);
        make_ready(t0, p0, c);
        tb = fetch();
        load_pair(tb, pb);
        ta = fetch();
    }

    XrDirT<NW> dir;
    XdRec rec{0, 0, 0, 0, 0u, 0u};
    uint32_t task = 0;
    const uint8_t *V = nullptr, *Hs = nullptr;
    int m = 0, n = 0, bv = 0, ev = 0, bh = 0, eh = 0;
    int phase = 0;     // 0: start a task, 1: left direction running, 2: right direction running
    auto write_rec = [&]() {
        if (rec.flags & XF_OVF) {
            rec.cells = 0;
            const unsigned int slot = atomicAdd(&kp.counter[2], 1u);
            kp.ovf[slot] = task;
        } else if (!(rec.flags & (XF_NONE | XF_SAME | XF_BADIDX))) {
            rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev;
            rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
            exec += rec.cells;
        }
        kp.xd[task] = rec;
    };
    for (;;) {
        while (phase == 0) {
            if (!(c.flags & XFT_VALID)) break;
            const XfReady cur = c;
            make_ready(tb, pb, c);
            tb = ta;
            load_pair(tb, pb);
            ta = fetch();
            task = cur.t;
            const int s = (int)(task & 1);
            rec = XdRec{0, 0, 0, 0, 0u, 0u};
            if (!(cur.flags & XFT_IDX)) {
                rec.flags = XF_BADIDX;
            } else if (s >= kp.seed_count ||
                       (s == 1 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && (cur.flags & XFT_FEW))) {
                rec.flags = XF_NONE;
            } else if (s == 1 && (cur.flags & XFT_SAME)) {
                rec.flags = XF_SAME;
            } else {
                V = kp.rseq + cur.r0; m = (int)(cur.r1 - cur.r0);
                Hs = kp.cseq + cur.c0; n = (int)(cur.c1 - cur.c0);
                bv = (int)(cur.seed & 0xffffu); bh = (int)(cur.seed >> 16);
                ev = bv + kp.seed_len; eh = bh + kp.seed_len;
                if (ev > m || eh > n) {
                    bv = min(bv, m); ev = min(ev, m); bh = min(bh, n); eh = min(eh, n);
                    rec.flags |= XF_BAD;
                }
                if (bv > 0 && bh > 0) {
                    dir.init(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1, kp.xg, kp.xdrop);
                    phase = 1;
                } else if (ev < m && eh < n) {
                    dir.init(V + ev, m - ev, 1, Hs + eh, n - eh, 1, kp.xg, kp.xdrop);
                    phase = 2;
                }
            }
            if (phase == 0) write_rec();
        }
        if (phase == 0) break;
        if (dir.step(tbl, kp.xg, kp.xdrop)) continue;
        const XdOut x = dir.finish();
        rec.cells += x.cells;
        if (!x.ok) {
            rec.flags |= XF_OVF;
            write_rec();
            phase = 0;
        } else if (phase == 1) {
            bv -= x.dv; bh -= x.dh;
            if (ev < m && eh < n) {
                dir.init(V + ev, m - ev, 1, Hs + eh, n - eh, 1, kp.xg, kp.xdrop);
                phase = 2;
            } else {
                write_rec();
                phase = 0;
            }
        } else {
            ev += x.dv; eh += x.dh;
            write_rec();
            phase = 0;
        }
    }
    if (exec) atomicAdd(kp.exec_cells, exec);
}

// ------------------------------------------------------------- k_xd_wide
__device__ __forceinline__ XdOut xdrop_dir_any(const uint8_t *V, int nv, int vstep,
                                               const uint8_t *Hs, int nh, int hstep,
                                               const int *ssm, int g, int X, int *sring,
                                               int *gring, int gring_w)
{
    XdOut o = xdrop_dir_warp(V, nv, vstep, Hs, nh, hstep, ssm, g, X, sring, RING_W);
    if (!o.ok) o = xdrop_dir_warp(V, nv, vstep, Hs, nh, hstep, ssm, g, X, gring, gring_w);
    return o;
}

// ------------------------------------------------------------------ k_xd16
// The extension in 16-bit lanes (xdrop_dir_thread16), a task per thread run to
// its end: two band cells per instruction.
// A task whose band outgrows the ring or whose score passes SAT16 goes to the
// overflow list and k_xd_wide reruns it in 32 bits.
__global__ void __launch_bounds__(XT) k_xd16(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    __shared__ uint32_t ring[3 * 8 * XT];
    load_sm(ssm, kp.sm);
    __syncthreads();
    uint32_t *base = ring + threadIdx.x;
    const uint64_t ntask = 2 * kp.n;
    unsigned long long exec = 0;
    for (;;) {
        const uint64_t task = atomicAdd(&kp.counter[1], 1u);
        if (task >= ntask) break;
        const uint64_t p = task >> 1;
        const int s = (int)(task & 1);
        const pg_pair pr = kp.pairs[p];
        XdRec rec{0, 0, 0, 0, 0u, 0u};
        const uint8_t *V, *Hs;
        int m, n;
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            rec.flags = XF_BADIDX;
        } else if (s >= kp.seed_count ||
                   (s == 1 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && pr.count < 2)) {
            rec.flags = XF_NONE;
        } else if (s == 1 && pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0) {
            rec.flags = XF_SAME;
        } else {
            int bv, ev, bh, eh;
            if (seed_region(kp, pr, s, m, n, bv, ev, bh, eh)) rec.flags |= XF_BAD;
            bool ok = true;
            if (bv > 0 && bh > 0) {
                const XdOut x = xdrop_dir_thread16<XT>(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1,
                                                       ssm, kp.xg, kp.xdrop, base);
                ok = x.ok; rec.cells += x.cells; bv -= x.dv; bh -= x.dh;
            }
            if (ok && ev < m && eh < n) {
                const XdOut x = xdrop_dir_thread16<XT>(V + ev, m - ev, 1, Hs + eh, n - eh, 1,
                                                       ssm, kp.xg, kp.xdrop, base);
                ok = x.ok; rec.cells += x.cells; ev += x.dv; eh += x.dh;
            }
            if (ok) {
                rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev; rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
                exec += rec.cells;
            } else {
                rec.flags |= XF_OVF;
                rec.cells = 0;
                const unsigned int slot = atomicAdd(&kp.counter[2], 1u);
                kp.ovf[slot] = (uint32_t)task;
            }
        }
        kp.xd[task] = rec;
    }
    if (exec) atomicAdd(kp.exec_cells, exec);   // index 0 = X-drop cells
}

// ------------------------------------------------------------------ k_xda
// The affine gap model of the extension (PG_F_XDROP_AFFINE): a warp per
// (pair, seed) task taken from the work counter, both directions by
// xdrop_dir_warp_affine on the warp's ring of 7 x gring_w ints in global
// memory (L2-resident; gring_w covers the longest sequence, so no band
// overflows).
__global__ void __launch_bounds__(WARPS * 32) k_xda(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + wib;
    int *ring = kp.gring + gw * (uint64_t)XDA_ARRAYS * (uint64_t)kp.gring_w;
    const uint64_t ntask = 2 * kp.n;
    unsigned long long exec = 0;
    for (;;) {
        unsigned int tk = 0;
        if (lane == 0) tk = atomicAdd(&kp.counter[1], 1u);
        const uint64_t task = __shfl_sync(FULL, tk, 0);
        if (task >= ntask) break;
        const uint64_t p = task >> 1;
        const int s = (int)(task & 1);
        const pg_pair pr = kp.pairs[p];
        XdRec rec{0, 0, 0, 0, 0u, 0u};
        const uint8_t *V, *Hs;
        int m, n;
        if (!pair_seqs(kp, pr, V, m, Hs, n)) {
            rec.flags = XF_BADIDX;
        } else if (s >= kp.seed_count ||
                   (s == 1 && (kp.flags & PG_F_SKIP_SPURIOUS_SEED) && pr.count < 2)) {
            rec.flags = XF_NONE;
        } else if (s == 1 && pr.rs1 == pr.rs0 && pr.cs1 == pr.cs0) {
            rec.flags = XF_SAME;
        } else {
            int bv, ev, bh, eh;
            if (seed_region(kp, pr, s, m, n, bv, ev, bh, eh)) rec.flags |= XF_BAD;
            if (bv > 0 && bh > 0) {
                const XdOut x = xdrop_dir_warp_affine(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1, ssm,
                                                      kp.go, kp.ge, kp.xdrop, ring, kp.gring_w);
                rec.cells += x.cells;
                bv -= x.dv; bh -= x.dh;
            }
            if (ev < m && eh < n) {
                const XdOut x = xdrop_dir_warp_affine(V + ev, m - ev, 1, Hs + eh, n - eh, 1, ssm,
                                                      kp.go, kp.ge, kp.xdrop, ring, kp.gring_w);
                rec.cells += x.cells;
                ev += x.dv; eh += x.dh;
            }
            rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev; rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
            exec += rec.cells;
        }
        if (lane == 0) kp.xd[task] = rec;
        __syncwarp();
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells, exec);
}

__global__ void __launch_bounds__(WARPS * 32) k_xd_wide(const KParams kp)
{
    __shared__ int ssm[32 * 32];
    __shared__ int sring[WARPS][3 * RING_W];
    load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t gw = (uint64_t)blockIdx.x * WARPS + wib;
    const uint64_t nw = (uint64_t)gridDim.x * WARPS;
    int *gring = kp.gring + gw * 3ull * (uint64_t)kp.gring_w;
    const unsigned int novf = kp.counter[2];
    unsigned long long exec = 0;
    for (uint64_t q = gw; q < novf; q += nw) {
        const uint32_t task = kp.ovf[q];
        const uint64_t p = task >> 1;
        const int s = (int)(task & 1);
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        pair_seqs(kp, pr, V, m, Hs, n);
        XdRec rec{0, 0, 0, 0, 0u, 0u};
        int bv, ev, bh, eh;
        if (seed_region(kp, pr, s, m, n, bv, ev, bh, eh)) rec.flags |= XF_BAD;
        if (bv > 0 && bh > 0) {
            const XdOut x = xdrop_dir_any(V + bv - 1, bv, -1, Hs + bh - 1, bh, -1, ssm, kp.xg,
                                          kp.xdrop, sring[wib], gring, kp.gring_w);
            rec.cells += x.cells;
            bv -= x.dv; bh -= x.dh;
        }
        if (ev < m && eh < n) {
            const XdOut x = xdrop_dir_any(V + ev, m - ev, 1, Hs + eh, n - eh, 1, ssm, kp.xg,
                                          kp.xdrop, sring[wib], gring, kp.gring_w);
            rec.cells += x.cells;
            ev += x.dv; eh += x.dh;
        }
        rec.bv = (uint16_t)bv; rec.ev = (uint16_t)ev; rec.bh = (uint16_t)bh; rec.eh = (uint16_t)eh;
        exec += rec.cells;
        if (lane == 0) kp.xd[task] = rec;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells, exec);
}

}  // namespace pg
