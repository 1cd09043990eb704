// pg_xdrop.cuh -- warp-level gapped X-drop extension (sm_103a).
//
// Restates seqan::extendSeed(seed, H, V, EXTEND_BOTH, score, x, GappedXDrop())
// as PASTIS calls it (src/align/SeqanXdropAligner.cpp:281-283), one direction
// at a time, by anti-diagonals of the (V consumed = column, H consumed = row)
// grid with a linear gap g:
//   T(c, r) = max(T(c-1, r) + g, T(c, r-1) + g, T(c-1, r-1) + s)
// A cell below best - X is dead; best is the maximum over completed
// anti-diagonals.  The band [lo, hi) of computed columns is trimmed of dead
// cells at both ends (current and previous anti-diagonal), widened by one on
// the right and clipped to the grid; the extension stops when it is empty.
// End point: the far corner if alive, else a fixed probe of the previous
// anti-diagonal, else the first maximum two anti-diagonals back.
//
// The three live anti-diagonals sit in a ring of W ints each (column c at slot
// c & (W-1)); lanes own consecutive columns of the band.  A band wider than the
// ring makes the routine report overflow so the caller can rerun the direction
// with a larger ring.
#pragma once
#include <cstdint>

#include "pg_dp.cuh"

namespace pg {

constexpr int UND = NEG;  // dead cell

struct XdOut {
    int dv, dh;        // residues consumed in V and in H
    uint32_t cells;    // band cells computed
    int ok;            // 0: ring overflow
};

// V / Hs point at the first residue to consume; vstep / hstep are +1 or -1.
__device__ inline XdOut xdrop_dir_warp(const uint8_t *__restrict__ V, int nv, int vstep,
                                const uint8_t *__restrict__ Hs, int nh, int hstep,
                                const int *__restrict__ ssm, int g, int X,
                                int *ring, int W)
{
    const int lane = threadIdx.x & 31;
    XdOut o{0, 0, 0u, 1};
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return o;
    const int mask = W - 1;
    int *A1 = ring, *A2 = ring + W, *A3 = ring + 2 * W;
    int off1 = 0, len1 = 0, off2 = 0, len2 = 1, off3 = 0, len3 = 2;
    if (lane == 0) {
        A2[0] = 0;
        const int v1 = (-g > X) ? UND : g;
        A3[0] = v1;
        A3[1] = v1;
    }
    __syncwarp();
    int best = 0, d = 1, lo = 1, hi = 2;
    while (lo < hi) {
        ++d;
        int *t = A1; A1 = A2; A2 = A3; A3 = t;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > W) { o.ok = 0; return o; }
        const int thr = best - X;
        int lbest = d * g;
        for (int c = lo + lane; c < hi; c += 32) {
            const int r = d - c;
            int v = max(A2[(c - 1) & mask], A2[c & mask]) + g;
            const int vr = __ldg(V + vstep * (c - 1));
            const int hr = __ldg(Hs + hstep * (r - 1));
            const int dg = A1[(c - 1) & mask] + ssm[vr * 32 + hr];
            v = max(v, dg);
            const bool live = v >= thr;
            A3[c & mask] = live ? v : UND;
            if (live) lbest = max(lbest, v);
        }
        if (lane == 0) {
            const int bval = (d * g > best - X) ? d * g : UND;
            A3[off3 & mask] = (off3 == 0) ? bval : UND;
            A3[hi & mask] = (d == hi && hi < cols) ? bval : UND;
        }
        __syncwarp();
        const int db = __reduce_max_sync(FULL, lbest);
        if (db > best) best = db;
        o.cells += (uint32_t)(hi - lo);
        // advance lo past columns whose cell and left predecessor are dead
        for (int c0 = lo;; c0 += 32) {
            const int c = c0 + lane;
            bool cond = (c - off3 < len3);
            if (cond) cond = A3[c & mask] == UND;
            if (cond) cond = (c - off2 - 1 < len2);
            if (cond) cond = A2[(c - 1) & mask] == UND;
            const unsigned bal = __ballot_sync(FULL, !cond);
            if (bal) { lo = c0 + __ffs(bal) - 1; break; }
        }
        // pull hi back over dead columns
        for (int c0 = hi;; c0 -= 32) {
            const int c = c0 - lane;
            bool cond = (c - off3 > 0);
            if (cond) cond = A3[(c - 1) & mask] == UND;
            if (cond) cond = A2[(c - 1) & mask] == UND;
            const unsigned bal = __ballot_sync(FULL, !cond);
            if (bal) { hi = c0 - (__ffs(bal) - 1); break; }
        }
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
        __syncwarp();
    }

    int lc = off3 + len3 - 2, lr = d - lc, ls = A3[lc & mask];
    if (ls == UND) {
        const int ca = off2 + len2 - 2;
        if (A2[ca & mask] != UND) {
            lc = ca; lr = d - 1 - lc; ls = A2[ca & mask];
        } else if (len2 > 2 && A2[(ca - 1) & mask] != UND) {
            lc = ca - 1; lr = d - 1 - lc; ls = A2[(ca - 1) & mask];
        }
    }
    if (ls == UND) {
        int bv = UND, bc = 0x7fffffff;
        for (int k = lane; k < len1; k += 32) {
            const int val = A1[(off1 + k) & mask];
            if (val > bv) { bv = val; bc = off1 + k; }
        }
        const int mv = __reduce_max_sync(FULL, bv);
        const unsigned cand = (bv == mv) ? (unsigned)bc : 0x7fffffffu;
        const int mc = (int)__reduce_min_sync(FULL, cand);
        if (mv != UND) { ls = mv; lc = mc; lr = d - 2 - lc; }
    }
    if (ls != UND) { o.dv = lc; o.dh = lr; }
    __syncwarp();
    return o;
}

// The affine gap model of the extension (PG_F_XDROP_AFFINE), a warp per
// direction: Gotoh's three states over the same anti-diagonals, a gap of
// length L scoring go + (L-1)*ge,
//   E(c, r) = max(T(c-1, r) + go, E(c-1, r) + ge)     (V consumed)
//   F(c, r) = max(T(c, r-1) + go, F(c, r-1) + ge)     (H consumed)
//   T(c, r) = max(T(c-1, r-1) + s, E(c, r), F(c, r))
// with a dead T killing all three states; the border cell of anti-diagonal d
// scores go + (d-1)*ge.  Band trimming and the end point are those of
// xdrop_dir_warp.  The ring holds 7 arrays of W ints (T for three
// anti-diagonals, E and F for two); W must cover the widest band (the caller
// passes a power of two at least the longer sequence + 4).
__device__ inline XdOut xdrop_dir_warp_affine(const uint8_t *__restrict__ V, int nv, int vstep,
                                              const uint8_t *__restrict__ Hs, int nh, int hstep,
                                              const int *__restrict__ ssm, int go, int ge, int X,
                                              int *ring, int W)
{
    const int lane = threadIdx.x & 31;
    XdOut o{0, 0, 0u, 1};
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return o;
    const int mask = W - 1;
    int *A1 = ring, *A2 = ring + W, *A3 = ring + 2 * W;
    int *E2 = ring + 3 * W, *E3 = ring + 4 * W, *F2 = ring + 5 * W, *F3 = ring + 6 * W;
    int off1 = 0, len1 = 0, off2 = 0, len2 = 1, off3 = 0, len3 = 2;
    if (lane == 0) {
        A2[0] = 0;
        const int v1 = (-go > X) ? UND : go;
        A3[0] = v1; A3[1] = v1;
        E3[0] = UND; F3[0] = v1;     // (0, 1): a gap along H
        E3[1] = v1; F3[1] = UND;     // (1, 0): a gap along V
    }
    __syncwarp();
    int best = 0, d = 1, lo = 1, hi = 2;
    while (lo < hi) {
        ++d;
        int *t = A1; A1 = A2; A2 = A3; A3 = t;
        t = E2; E2 = E3; E3 = t;
        t = F2; F2 = F3; F3 = t;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > W) { o.ok = 0; return o; }
        const int thr = best - X;
        const long long bs = (long long)go + (long long)(d - 1) * ge;
        const int bscore = bs < UND ? UND : (int)bs;
        int lbest = bscore;
        for (int c = lo + lane; c < hi; c += 32) {
            const int r = d - c;
            const int e = max(A2[(c - 1) & mask] + go, E2[(c - 1) & mask] + ge);
            const int f = max(A2[c & mask] + go, F2[c & mask] + ge);
            const int vr = __ldg(V + vstep * (c - 1));
            const int hr = __ldg(Hs + hstep * (r - 1));
            const int v = max(A1[(c - 1) & mask] + ssm[vr * 32 + hr], max(e, f));
            const bool live = v >= thr;
            A3[c & mask] = live ? v : UND;
            E3[c & mask] = live ? e : UND;
            F3[c & mask] = live ? f : UND;
            if (live) lbest = max(lbest, v);
        }
        if (lane == 0) {
            const int bval = ((long long)bscore > (long long)best - X) ? bscore : UND;
            const int lo_t = (off3 == 0) ? bval : UND;
            A3[off3 & mask] = lo_t; E3[off3 & mask] = UND; F3[off3 & mask] = lo_t;
            const int hi_t = (d == hi && hi < cols) ? bval : UND;
            A3[hi & mask] = hi_t; E3[hi & mask] = hi_t; F3[hi & mask] = UND;
        }
        __syncwarp();
        const int db = __reduce_max_sync(FULL, lbest);
        if (db > best) best = db;
        o.cells += (uint32_t)(hi - lo);
        for (int c0 = lo;; c0 += 32) {
            const int c = c0 + lane;
            bool cond = (c - off3 < len3);
            if (cond) cond = A3[c & mask] == UND;
            if (cond) cond = (c - off2 - 1 < len2);
            if (cond) cond = A2[(c - 1) & mask] == UND;
            const unsigned bal = __ballot_sync(FULL, !cond);
            if (bal) { lo = c0 + __ffs(bal) - 1; break; }
        }
        for (int c0 = hi;; c0 -= 32) {
            const int c = c0 - lane;
            bool cond = (c - off3 > 0);
            if (cond) cond = A3[(c - 1) & mask] == UND;
            if (cond) cond = A2[(c - 1) & mask] == UND;
            const unsigned bal = __ballot_sync(FULL, !cond);
            if (bal) { hi = c0 - (__ffs(bal) - 1); break; }
        }
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
        __syncwarp();
    }

    int lc = off3 + len3 - 2, lr = d - lc, ls = A3[lc & mask];
    if (ls == UND) {
        const int ca = off2 + len2 - 2;
        if (A2[ca & mask] != UND) {
            lc = ca; lr = d - 1 - lc; ls = A2[ca & mask];
        } else if (len2 > 2 && A2[(ca - 1) & mask] != UND) {
            lc = ca - 1; lr = d - 1 - lc; ls = A2[(ca - 1) & mask];
        }
    }
    if (ls == UND) {
        int bv = UND, bc = 0x7fffffff;
        for (int k = lane; k < len1; k += 32) {
            const int val = A1[(off1 + k) & mask];
            if (val > bv) { bv = val; bc = off1 + k; }
        }
        const int mv = __reduce_max_sync(FULL, bv);
        const unsigned cand = (bv == mv) ? (unsigned)bc : 0x7fffffffu;
        const int mc = (int)__reduce_min_sync(FULL, cand);
        if (mv != UND) { ls = mv; lc = mc; lr = d - 2 - lc; }
    }
    if (ls != UND) { o.dv = lc; o.dh = lr; }
    __syncwarp();
    return o;
}

// The same extension run by one thread from start to end (k_xd).  The ring
// holds W ints per
// anti-diagonal; slot (array k, column c) sits at base[(k*W + (c & (W-1))) * NT]
// where base = ring + threadIdx.x, so the 32 lanes of a warp always touch 32
// different banks.  Bands wider than W report overflow (ok = 0).
template <int W, int NT>
__device__ __forceinline__ XdOut xdrop_dir_thread(const uint8_t *__restrict__ V, int nv, int vstep,
                                                  const uint8_t *__restrict__ Hs, int nh, int hstep,
                                                  const int *__restrict__ ssm, int g, int X,
                                                  int *__restrict__ base)
{
    XdOut o{0, 0, 0u, 1};
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return o;
#define RING(k, c) base[((k) * W + ((c) & (W - 1))) * NT]
    int k1 = 0, k2 = 1, k3 = 2;
    int off1 = 0, len1 = 0, off2 = 0, len2 = 1, off3 = 0, len3 = 2;
    RING(k2, 0) = 0;
    {
        const int v1 = (-g > X) ? UND : g;
        RING(k3, 0) = v1;
        RING(k3, 1) = v1;
    }
    int best = 0, d = 1, lo = 1, hi = 2;
    while (lo < hi) {
        ++d;
        const int kt = k1; k1 = k2; k2 = k3; k3 = kt;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > W) { o.ok = 0; return o; }
        const int thr = best - X;
        {
            const int bval = (d * g > best - X) ? d * g : UND;
            RING(k3, off3) = (off3 == 0) ? bval : UND;
            RING(k3, hi) = (d == hi && hi < cols) ? bval : UND;
        }
        int dbest = d * g;
        int a2prev = RING(k2, lo - 1);
        const uint8_t *vp = V + vstep * (lo - 1);
        const uint8_t *hp = Hs + hstep * (d - lo - 1);
        for (int c = lo; c < hi; ++c) {
            const int a2c = RING(k2, c);
            int v = max(a2prev, a2c) + g;
            const int dg = RING(k1, c - 1) + ssm[(int)__ldg(vp) * 32 + (int)__ldg(hp)];
            v = max(v, dg);
            const bool live = v >= thr;
            RING(k3, c) = live ? v : UND;
            if (live) dbest = max(dbest, v);
            a2prev = a2c;
            vp += vstep;
            hp -= hstep;
        }
        if (dbest > best) best = dbest;
        o.cells += (uint32_t)(hi - lo);
        while (lo - off3 < len3 && RING(k3, lo) == UND && lo - off2 - 1 < len2 && RING(k2, lo - 1) == UND)
            ++lo;
        while (hi - off3 > 0 && RING(k3, hi - 1) == UND && RING(k2, hi - 1) == UND)
            --hi;
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
    }
    int lc = off3 + len3 - 2, lr = d - lc, ls = RING(k3, lc);
    if (ls == UND) {
        const int ca = off2 + len2 - 2;
        if (RING(k2, ca) != UND) {
            lc = ca; lr = d - 1 - lc; ls = RING(k2, ca);
        } else if (len2 > 2 && RING(k2, ca - 1) != UND) {
            lc = ca - 1; lr = d - 1 - lc; ls = RING(k2, ca - 1);
        }
    }
    if (ls == UND) {
        for (int k = 0; k < len1; ++k) {
            const int val = RING(k1, off1 + k);
            if (val > ls) { ls = val; lc = off1 + k; lr = d - 2 - lc; }
        }
    }
#undef RING
    if (ls != UND) { o.dv = lc; o.dh = lr; }
    return o;
}

// xdrop_dir_thread cut at anti-diagonal bounds so that a caller can step one
// direction at a time and start another the moment one ends (k_xdf), on the
// same ring.
// init sets up a direction of at least one residue on each side; step
// computes one anti-diagonal and returns whether the direction goes on (false
// also when the band outgrows the ring: ok = 0); finish gives its end point.
template <int W, int NT>
struct XdDir {
    const uint8_t *V, *Hs;
    int vstep, hstep, cols, rows;
    int k1, k2, k3, off1, len1, off2, len2, off3, len3;
    int best, d, lo, hi, ok;
    uint32_t cells;
    int vr0, hr0;        // residues of the band's first cell on the next anti-diagonal

#define XRING(k, c) base[((k) * W + ((c) & (W - 1))) * NT]
    __device__ __forceinline__ void init(const uint8_t *V_, int nv, int vstep_, const uint8_t *Hs_, int nh,
                                         int hstep_, int g, int X, int *base)
    {
        V = V_; Hs = Hs_; vstep = vstep_; hstep = hstep_;
        cols = nv + 1; rows = nh + 1;
        k1 = 0; k2 = 1; k3 = 2;
        off1 = 0; len1 = 0; off2 = 0; len2 = 1; off3 = 0; len3 = 2;
        XRING(k2, 0) = 0;
        const int v1 = (-g > X) ? UND : g;
        XRING(k3, 0) = v1;
        XRING(k3, 1) = v1;
        best = 0; d = 1; lo = 1; hi = 2; ok = 1; cells = 0;
        vr0 = __ldg(V);                 // anti-diagonal 2 starts at column 1, row 1
        hr0 = __ldg(Hs);
    }
    __device__ __forceinline__ bool step(const int *__restrict__ ssm, int g, int X, int *base)
    {
        ++d;
        const int kt = k1; k1 = k2; k2 = k3; k3 = kt;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > W) { ok = 0; return false; }
        const int thr = best - X;
        {
            const int bval = (d * g > best - X) ? d * g : UND;
            XRING(k3, off3) = (off3 == 0) ? bval : UND;
            XRING(k3, hi) = (d == hi && hi < cols) ? bval : UND;
        }
        int dbest = d * g;
        int a2prev = XRING(k2, lo - 1);
        const uint8_t *vp = V + vstep * (lo - 1);
        const uint8_t *hp = Hs + hstep * (d - lo - 1);
        // residues are read one cell ahead (and the first cell's a step ahead)
        int vr = vr0, hr = hr0;
        for (int c = lo; c < hi; ++c) {
            vp += vstep;
            hp -= hstep;
            int vn = 0, hn = 0;
            if (c + 1 < hi) { vn = __ldg(vp); hn = __ldg(hp); }
            const int a2c = XRING(k2, c);
            int v = max(a2prev, a2c) + g;
            const int dg = XRING(k1, c - 1) + ssm[vr * 32 + hr];
            v = max(v, dg);
            const bool live = v >= thr;
            XRING(k3, c) = live ? v : UND;
            if (live) dbest = max(dbest, v);
            a2prev = a2c;
            vr = vn; hr = hn;
        }
        if (dbest > best) best = dbest;
        cells += (uint32_t)(hi - lo);
        while (lo - off3 < len3 && XRING(k3, lo) == UND && lo - off2 - 1 < len2 && XRING(k2, lo - 1) == UND)
            ++lo;
        while (hi - off3 > 0 && XRING(k3, hi - 1) == UND && XRING(k2, hi - 1) == UND)
            --hi;
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
        if (lo < hi) {
            // the next anti-diagonal (d + 1) starts at column lo: V[lo - 1], H[d - lo]
            vr0 = __ldg(V + vstep * (lo - 1));
            hr0 = __ldg(Hs + hstep * (d - lo));
        }
        return lo < hi;
    }
    __device__ __forceinline__ XdOut finish(const int *base) const
    {
        XdOut o{0, 0, cells, ok};
        if (!ok) return o;
        int lc = off3 + len3 - 2, lr = d - lc, ls = XRING(k3, lc);
        if (ls == UND) {
            const int ca = off2 + len2 - 2;
            if (XRING(k2, ca) != UND) {
                lc = ca; lr = d - 1 - lc; ls = XRING(k2, ca);
            } else if (len2 > 2 && XRING(k2, ca - 1) != UND) {
                lc = ca - 1; lr = d - 1 - lc; ls = XRING(k2, ca - 1);
            }
        }
        if (ls == UND) {
            for (int k = 0; k < len1; ++k) {
                const int val = XRING(k1, off1 + k);
                if (val > ls) { ls = val; lc = off1 + k; lr = d - 2 - lc; }
            }
        }
        if (ls != UND) { o.dv = lc; o.dh = lr; }
        return o;
    }
#undef XRING
};

// ------------------------------------------------------------------------
// The per-thread extension in 16-bit lanes, two band cells per instruction
// (__vmaxs2 / __vaddss2 / __vcmpges2 on int16x2).  A live cell lies in
// [best - X, best + max score], so 16 bits hold every live value while
// best <= SAT16 and X <= XMAX16; when best passes SAT16 the routine stops and
// reports ok = 0 (as for a band wider than the ring) and the caller reruns
// the extension in 32 bits.  Whenever it completes its result equals
// the 32-bit extension's.  Ring: 3 arrays x 8 words (16 int16 slots, column c at
// half c & 1 of word (c >> 1) & 7), word (k, j) at wbase[(k * 8 + j) * NT].
constexpr int UND16 = -32768;
constexpr int SAT16 = 30000;
constexpr int XMAX16 = 30000;

template <int NT>
__device__ __forceinline__ XdOut xdrop_dir_thread16(const uint8_t *__restrict__ V, int nv, int vstep,
                                                    const uint8_t *__restrict__ Hs, int nh, int hstep,
                                                    const int *__restrict__ ssm, int g, int X,
                                                    uint32_t *__restrict__ wbase)
{
    XdOut o{0, 0, 0u, 1};
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return o;
#define WD(k, j) wbase[((k) * 8 + ((j) & 7)) * NT]
#define HW(k, c) reinterpret_cast<int16_t *>(&WD(k, (c) >> 1))[(c) & 1]
    int k1 = 0, k2 = 1, k3 = 2;
    int off1 = 0, len1 = 0, off2 = 0, len2 = 1, off3 = 0, len3 = 2;
    HW(k2, 0) = 0;
    {
        const int v1 = (-g > X) ? UND16 : g;
        HW(k3, 0) = (int16_t)v1;
        HW(k3, 1) = (int16_t)v1;
    }
    const uint32_t g2 = (uint32_t)(g & 0xffff) * 0x10001u;
    int best = 0, d = 1, lo = 1, hi = 2;
    while (lo < hi) {
        ++d;
        const int kt = k1; k1 = k2; k2 = k3; k3 = kt;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > 16 || best > SAT16) { o.ok = 0; return o; }
        const int thr = best - X;
        {
            const int bval = (d * g > best - X) ? d * g : UND16;
            HW(k3, off3) = (int16_t)((off3 == 0) ? bval : UND16);
            HW(k3, hi) = (int16_t)((d == hi && hi < cols) ? bval : UND16);
        }
        const uint32_t thr2 = (uint32_t)(thr & 0xffff) * 0x10001u;
        uint32_t db2 = 0x80008000u;
        const int j0 = lo >> 1, j1 = (hi - 1) >> 1;
        uint32_t a2p = WD(k2, j0 - 1), a1p = WD(k1, j0 - 1);
        for (int j = j0; j <= j1; ++j) {
            const int c0 = 2 * j, c1 = c0 + 1;
            const uint32_t a2 = WD(k2, j), a1 = WD(k1, j);
            uint32_t v = __vaddss2(__vmaxs2(__byte_perm(a2p, a2, 0x5432), a2), g2);
            // residues V[c-1], H[d-c-1]; a half outside [lo, hi) reads a clamped
            // index and is discarded below
            const int vi0 = c0 - 1 > 0 ? c0 - 1 : 0;
            const int vi1 = c1 - 1 < nv - 1 ? c1 - 1 : nv - 1;
            // (a discarded low half c0 = lo - 1 can ask for H[nh], one past the end)
            const int hi0 = d - c0 - 1 < nh - 1 ? d - c0 - 1 : nh - 1;
            const int hi1 = d - c1 - 1 > 0 ? d - c1 - 1 : 0;
            const int s0 = ssm[(int)__ldg(V + vstep * vi0) * 32 + (int)__ldg(Hs + hstep * hi0)];
            const int s1 = ssm[(int)__ldg(V + vstep * vi1) * 32 + (int)__ldg(Hs + hstep * hi1)];
            const uint32_t s2 = __byte_perm((uint32_t)s0, (uint32_t)s1, 0x5410);
            v = __vmaxs2(v, __vaddss2(__byte_perm(a1p, a1, 0x5432), s2));
            const uint32_t live = __vcmpges2(v, thr2);
            v = (v & live) | (0x80008000u & ~live);
            uint32_t keep = 0;
            if (c0 < lo) keep |= 0x0000ffffu;
            if (c1 >= hi) keep |= 0xffff0000u;
            if (keep) v = (v & ~keep) | (WD(k3, j) & keep);
            WD(k3, j) = v;
            db2 = __vmaxs2(db2, v);
            a2p = a2;
            a1p = a1;
        }
        int dbest = d * g;
        const int m0 = (int)(int16_t)(db2 & 0xffffu), m1 = (int)(int16_t)(db2 >> 16);
        dbest = max(dbest, max(m0, m1));
        if (dbest > best) best = dbest;
        o.cells += (uint32_t)(hi - lo);
        while (lo - off3 < len3 && HW(k3, lo) == UND16 && lo - off2 - 1 < len2 && HW(k2, lo - 1) == UND16)
            ++lo;
        while (hi - off3 > 0 && HW(k3, hi - 1) == UND16 && HW(k2, hi - 1) == UND16)
            --hi;
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
    }
    int lc = off3 + len3 - 2, lr = d - lc, ls = HW(k3, lc);
    if (ls == UND16) {
        const int ca = off2 + len2 - 2;
        if (HW(k2, ca) != UND16) {
            lc = ca; lr = d - 1 - lc; ls = HW(k2, ca);
        } else if (len2 > 2 && HW(k2, ca - 1) != UND16) {
            lc = ca - 1; lr = d - 1 - lc; ls = HW(k2, ca - 1);
        }
    }
    if (ls == UND16) {
        for (int q = 0; q < len1; ++q) {
            const int val = HW(k1, off1 + q);
            if (val > ls) { ls = val; lc = off1 + q; lr = d - 2 - lc; }
        }
    }
#undef HW
#undef WD
    if (ls != UND16) { o.dv = lc; o.dh = lr; }
    return o;
}

}  // namespace pg
