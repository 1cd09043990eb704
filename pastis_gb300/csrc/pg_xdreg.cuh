// pg_xdreg.cuh -- gapped X-drop extension with the band in registers (sm_103a).
//
// The same direction as xdrop_dir_thread (pg_xdrop.cuh), restating
// seqan::extendSeed(..., GappedXDrop()) as src/align/SeqanXdropAligner.cpp:281-283
// calls it, with identical band cells, end point and cell count, but with a
// different machine shape.  One thread holds a window of NS = 2 NW
// anti-diagonal columns in registers (k_xdr uses NW = 8: 16 columns): column c
// lives in slot c mod NS, two slots per 32-bit register (slot 2k in the low
// half, 2k+1 in the high half), as int16 values relative to a base B that
// moves up by RB when the best score passes B + RB.  Every step computes all
// NS slots with packed 16-bit max/add (two cells per instruction), without a
// branch on the band.  This is exact because a cell outside the band [lo, hi)
// always comes out dead:
//   - columns left of lo were trimmed (dead, with a dead left neighbour one
//     anti-diagonal back), columns right of hi have only dead predecessors,
//     cells with r < 0 have none; so the recurrence gives them nothing live;
//   - the band plus its two border columns spans at most NS - 1 slots, so
//     the slot left of the window (slot off3 - 1, which wraps to off3 + NS - 1)
//     never holds a live value; a wider window is reported as overflow;
//   - cells past either sequence end (c >= cols or r >= rows; column 0 is the
//     border and stays) are killed through their threshold each step, since
//     gap moves would carry live values there;
//   - the two border cells (column 0, row 0) come out as d * g from the
//     recurrence itself; only the reference's strict test (d * g > best - X,
//     where cells use >=) needs a rare fix, on equality.
// The live masks of the last two anti-diagonals give the next lo and hi with
// a few bit operations (the band trims), and the cell count is their sum.
// The residues: V per slot is static while the slot keeps its column (a fresh
// one is loaded for the column entering at hi); H moves one slot per step
// (the cell one column right on the next anti-diagonal has the same row) with
// a fresh one for the leftmost slot.  Scores come from a 25 x 33 int table in
// shared memory (row stride 33 spreads the banks) at byte offset
// V * 132 + H * 4, both offsets kept as 16-bit halves per slot pair.
//
// Requirements (otherwise the caller uses the ring kernel): linear gap
// -4096 <= g <= -1 and 0 <= X <= 8192, which keep every sum inside int16 with
// the dead value -16384.
#pragma once
#include <cstdint>

#include "pg_dpdir16.cuh"
#include "pg_xdrop.cuh"

namespace pg {

constexpr int XR_UND = -16384;                 // dead cell
constexpr uint32_t XR_UND2 = 0xC000C000u;
constexpr int XR_RB = 8192;                    // base step
constexpr int XR_TKILL = 12000;                // threshold of a killed slot (above every live value)
constexpr int XR_XMAX = 8192;
constexpr int XR_GMAX = 4096;
constexpr int XR_STRIDE = 33;                  // score table row stride (ints)
constexpr uint32_t XR_GARB_V = 24u * XR_STRIDE * 4u;   // offsets of a residue code that is in range
constexpr uint32_t XR_GARB_H = 24u * 4u;

__host__ __device__ __forceinline__ bool xdr_supported(int g, int X)
{
    return g <= -1 && g >= -XR_GMAX && X >= 0 && X <= XR_XMAX;
}

__device__ __forceinline__ void load_sm33(int *ssm, const int8_t *sm)
{
    for (int t = threadIdx.x; t < PG_NRES * XR_STRIDE; t += blockDim.x) {
        const int a = t / XR_STRIDE, b = t - a * XR_STRIDE;
        ssm[t] = b < PG_NRES ? (int)sm[a * PG_NRES + b] : 0;
    }
}

// Slot access at a runtime index.  Each register is tested with a predicated
// PTX instruction: written as plain C++ the compiler folds the eight tests
// back into an indexed array access, which puts the whole window in local
// memory.

// x mod NS for x >= 0
template <int NS>
__device__ __forceinline__ int xr_mod(int x)
{
    return NS == 16 ? (x & 15) : (int)((unsigned)x % (unsigned)NS);
}
// rotations of an NS-bit mask by s in [0, NS)
template <int NS>
__device__ __forceinline__ uint32_t xr_rotl(uint32_t m, int s)
{
    return ((m << s) | (m >> (NS - s))) & ((1u << NS) - 1u);
}
template <int NS>
__device__ __forceinline__ uint32_t xr_rotr(uint32_t m, int s)
{
    return ((m >> s) | (m << (NS - s))) & ((1u << NS) - 1u);
}

// the value of slot s (0..2NW-1) of a packed NW-register array
template <int NW>
__device__ __forceinline__ int xr_slot(const uint32_t (&R)[NW], int s)
{
    const int q = s >> 1;
    uint32_t w = R[0];
#pragma unroll
    for (int k = 1; k < NW; ++k)
        asm("{\n\t.reg .pred p;\n\tsetp.eq.s32 p, %1, %2;\n\t@p mov.b32 %0, %3;\n\t}"
            : "+r"(w) : "r"(q), "r"(k), "r"(R[k]));
    return (s & 1) ? hi16(w) : lo16(w);
}

// replace the half of slot s with the low half of x
template <int NW>
__device__ __forceinline__ void xr_put(uint32_t (&R)[NW], int s, uint32_t x)
{
    const uint32_t sel = (s & 1) ? 0x5410u : 0x3254u;
    const int q = s >> 1;
#pragma unroll
    for (int k = 0; k < NW; ++k)
        asm("{\n\t.reg .pred p;\n\tsetp.eq.s32 p, %1, %2;\n\t@p prmt.b32 %0, %0, %3, %4;\n\t}"
            : "+r"(R[k]) : "r"(q), "r"(k), "r"(x), "r"(sel));
}

template <int NW>
struct XrDirT {
    static constexpr int NS = 2 * NW;                 // window slots
    static constexpr uint32_t MASK = (1u << NS) - 1u;
    const uint8_t *V, *Hs;
    int vstep, hstep, nv, nh, cols, rows;
    uint32_t P[NW];    // anti-diagonal d - 1 (after a step: d)
    uint32_t L[NW];    // anti-diagonal d - 2 shifted one slot right (slot s holds column s - 1)
    uint32_t VO[NW];   // per slot: V code * 132 (score table row)
    uint32_t HO[NW];   // per slot: H code * 4
    uint32_t live2;    // slots of P that are live
    int off1, len1, off2, len2, off3, len3;
    int d, lo, hi, best, B, ok;   // best: the best score so far minus B
    uint32_t cells;
    uint32_t nv_off, nh_off;   // fresh residue offsets loaded for the next step
    // the last step's anti-diagonal d (the end rule reads it with P and L)
    uint32_t N[NW];
    uint32_t live3;

    // V / Hs point at the first residue to consume (at least one on each side)
    __device__ __forceinline__ void init(const uint8_t *V_, int nv_, int vstep_, const uint8_t *Hs_,
                                         int nh_, int hstep_, int g, int X)
    {
        V = V_; Hs = Hs_; vstep = vstep_; hstep = hstep_; nv = nv_; nh = nh_;
        cols = nv + 1; rows = nh + 1;
        const int v1 = (-g > X) ? XR_UND : g;
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            P[k] = XR_UND2; L[k] = XR_UND2; N[k] = XR_UND2;
            VO[k] = XR_GARB_V * 0x10001u; HO[k] = XR_GARB_H * 0x10001u;
        }
        P[0] = pk16(v1, v1);               // d = 1: columns 0 and 1
        L[0] = pk16(XR_UND, 0);            // d = 0 (column 0 = 0), shifted: slot 1 holds 0
        live2 = v1 == XR_UND ? 0u : 3u;
        off1 = 0; len1 = 0; off2 = 0; len2 = 1; off3 = 0; len3 = 2;
        d = 1; lo = 1; hi = 2; best = 0; B = 0; ok = 1; cells = 0;
        live3 = 0;
        // column 1 reads V[0]; column 0 at d = 1 reads H[0], which moves to column 1 at d = 2
        VO[0] = pk16((int)XR_GARB_V, (int)__ldg(V) * XR_STRIDE * 4);
        HO[0] = pk16((int)__ldg(Hs) * 4, (int)XR_GARB_H);
        // residues the end of step d = 2 inserts: H for column off3 = 0, V for column hi = 2
        nh_off = (nh > 1 ? (uint32_t)__ldg(Hs + hstep) : 24u) * 4u;
        nv_off = (nv > 1 ? (uint32_t)__ldg(V + vstep) : 24u) * (uint32_t)(XR_STRIDE * 4);
    }

    // one anti-diagonal; false when the direction ends (ok = 0: window overflow)
    __device__ __forceinline__ bool step(const char *__restrict__ tbl, int g, int X)
    {
        ++d;
        off1 = off2; len1 = len2;
        off2 = off3; len2 = len3;
        off3 = lo - 1; len3 = hi + 1 - off3;
        if (len3 > NS - 1) { ok = 0; return false; }
        const int thr = best - X;                 // best and the values are relative to B
        const uint32_t g2 = pk16(g, g);
        // H moves one slot: slot s takes slot s - 1 (the cell one column right
        // on this anti-diagonal has the row the left one had on the last)
        {
            uint32_t hl = HO[NW - 1];
#pragma unroll
            for (int k = NW - 1; k > 0; --k) HO[k] = prmt(HO[k - 1], HO[k], 0x5432u);
            HO[0] = prmt(hl, HO[0], 0x5432u);
        }
        // killed slots: c >= min(cols, d + 1) at the top of the window, and the
        // row past H at the bottom (which is off3 when the rows clamp holds it),
        // but not column 0
        uint32_t krel = 0;
        {
            const int top = min(cols, d + 1) - off3;
            if (top < NS) krel = (MASK << max(top, 0)) & MASK;
            if (off3 > 0 && off3 == d - rows) krel |= 1u;
        }
        const int sh = xr_mod<NS>(off3);
        const uint32_t kslot = xr_rotl<NS>(krel, sh);
        const uint32_t kp = (kslot | (kslot << 15)) & 0x55555555u;
        const uint32_t nthr2 = pk16(-thr, -thr);
        const uint32_t nkill2 = pk16(-XR_TKILL, -XR_TKILL);
        uint32_t lm = 0;
        uint32_t L2[NW];
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            const uint32_t pl = P[(k + NW - 1) % NW];
            L2[k] = prmt(pl, P[k], 0x5432u);           // slot s: column s - 1
            const uint32_t up = v16max(L2[k], P[k]);
            const uint32_t pair = VO[k] + HO[k];
            const int s0 = *reinterpret_cast<const int *>(tbl + (pair & 0xffffu));
            const int s1 = *reinterpret_cast<const int *>(tbl + (pair >> 16));
            const uint32_t s2 = prmt((uint32_t)s0, (uint32_t)s1, 0x5410u);
            const uint32_t dg = v16add(L[k], s2);
            const uint32_t v = __viaddmax_s16x2(up, g2, dg);
            const uint32_t mk = prmt(kp << (15 - 2 * k), 0u, 0xBB99u);
            const uint32_t nt = (nthr2 & ~mk) | (nkill2 & mk);
            const uint32_t t = v16add(v, nt);
            const uint32_t dead = prmt(t, 0u, 0xBB99u);
            N[k] = (v & ~dead) | (XR_UND2 & dead);
            lm |= ((~dead) >> (15 - 2 * k)) & (0x00010001u << (2 * k));
        }
        uint32_t live = (lm | (lm >> 15)) & MASK;
        // the reference keeps a border cell only when d * g > best - X
        if ((long long)d * g == (long long)(best + B) - X) {
            if (off3 == 0) { N[0] = prmt(N[0], XR_UND2, 0x3254u); live &= ~1u; }
            if (d - off3 < NS) {
                const int sd = xr_mod<NS>(d);
                xr_put(N, sd, XR_UND2);
                live &= ~(1u << sd);
            }
        }
        // best over the live cells (borders are d * g, which dbest starts from)
        int dbest = d * g;
        if (live) {
            const uint32_t m = vmax_all(N);
            const int mx = max(lo16(m), hi16(m)) + B;
            dbest = max(dbest, mx);
        }
        if (dbest > best + B) best = dbest - B;
        cells += (uint32_t)(hi - lo);
        // band trims from the live masks, in window order (bit p = column off3 + p)
        const uint32_t r3 = xr_rotr<NS>(live, sh), r2 = xr_rotr<NS>(live2, sh);
        const int span = hi - off3;            // 1..NS-2
        const uint32_t tl = (r3 | (r2 << 1)) & ~1u & ((2u << span) - 1u);
        const int lt = tl ? off3 + __ffs(tl) - 1 : hi + 1;
        const uint32_t tu = (r3 | r2) & ((1u << span) - 1u);
        const int ht = tu ? off3 + 32 - __clz(tu) : off3;
        const int hi_used = hi;
        const int off3_used = off3;
        lo = max(lt, d + 2 - rows);
        hi = min(ht + 1, cols);
        live3 = live;
        // residues loaded for this step go in now (used from the next step on)
        xr_put(HO, xr_mod<NS>(off3_used), nh_off);
        xr_put(VO, xr_mod<NS>(hi_used), nv_off);
        if (lo >= hi) return false;
        // fresh residues for the next step: H for its column off3, V for its column hi
        {
            const int no3 = lo - 1;
            const int hidx = d + 1 - no3 - 1;
            nh_off = (hidx >= 0 && hidx < nh ? (uint32_t)__ldg(Hs + hstep * hidx) : 24u) * 4u;
            const int vidx = hi - 1;
            nv_off = (vidx >= 0 && vidx < nv ? (uint32_t)__ldg(V + vstep * vidx) : 24u) *
                     (uint32_t)(XR_STRIDE * 4);
        }
        // rare: move the base so the values stay inside int16
        if (best > XR_RB) {
            const uint32_t rb2 = pk16(-XR_RB, -XR_RB);
#pragma unroll
            for (int k = 0; k < NW; ++k) {
                N[k] = v16max(v16add(N[k], rb2), XR_UND2);
                L2[k] = v16max(v16add(L2[k], rb2), XR_UND2);
            }
            best -= XR_RB;
            B += XR_RB;
        }
#pragma unroll
        for (int k = 0; k < NW; ++k) { L[k] = L2[k]; P[k] = N[k]; }
        live2 = live3;
        return true;
    }

    // end point after the last step (the rule of xdrop_dir_thread: the far
    // corner if alive, else a fixed probe of the previous anti-diagonal, else
    // the first maximum two anti-diagonals back)
    __device__ __forceinline__ XdOut finish() const
    {
        XdOut o{0, 0, cells, ok};
        if (!ok) return o;
        int lc = off3 + len3 - 2, lr = d - lc;
        int ls = xr_slot(N, xr_mod<NS>(lc));
        if (ls == XR_UND) {
            const int ca = off2 + len2 - 2;
            const int a0 = xr_slot(P, xr_mod<NS>(ca));
            if (a0 != XR_UND) {
                lc = ca; lr = d - 1 - lc; ls = a0;
            } else if (len2 > 2) {
                const int a1 = xr_slot(P, xr_mod<NS>(ca - 1));
                if (a1 != XR_UND) { lc = ca - 1; lr = d - 1 - lc; ls = a1; }
            }
        }
        if (ls == XR_UND) {
            // the first maximum of anti-diagonal d - 2 in column order.  Every
            // slot outside its window [off1, off1 + len1) is dead, so the
            // maximum over all slots is the window's; slot s of L holds column
            // s - 1, so column off1 + p sits at slot (off1 + 1 + p) mod NS.
            const uint32_t m = vmax_all(L);
            const int mx = max(lo16(m), hi16(m));
            if (mx != XR_UND) {
                const uint32_t m2 = pk16(mx, mx);
                uint32_t eq = 0;
#pragma unroll
                for (int k = 0; k < NW; ++k) {
                    const uint32_t e = __vcmpeq2(L[k], m2);
                    eq |= ((e & 1u) << (2 * k)) | (((e >> 16) & 1u) << (2 * k + 1));
                }
                const uint32_t w = xr_rotr<NS>(eq, xr_mod<NS>(off1 + 1)) & ((1u << len1) - 1u);
                if (w) { ls = mx; lc = off1 + __ffs(w) - 1; lr = d - 2 - lc; }
            }
        }
        if (ls != XR_UND) { o.dv = lc; o.dh = lr; }
        return o;
    }

    // the maximum of each half over the window's registers
    static __device__ __forceinline__ uint32_t vmax_all(const uint32_t (&R)[NW])
    {
        uint32_t m = R[0];
#pragma unroll
        for (int k = 1; k < NW; ++k) m = v16max(m, R[k]);
        return m;
    }
};

using XrDir = XrDirT<8>;

}  // namespace pg
