// pg_dpdir16.cuh -- the traceback-form DP on 16-bit lanes (sm_103a).
//
// dp_warp_dir (pg_dpdir.cuh) with each lane split into two virtual lanes held
// in the two halves of 32-bit registers: the low half works R rows, the high
// half the R rows below them one column behind.  A warp is a wavefront of 64
// virtual lanes (virtual lane v = 2 * lane + half works column k - v + 1 at
// step k), and each packed max / add (PTX max.s16x2, add.s16x2) computes two
// cells.  The high half's upper neighbour is the low half of the same lane one
// step earlier; the low half's is the high half of the lane above, handed down
// by one __shfl_up_sync of the packed edge.
//
// Scores are exact while every value of the region stays inside int16.  A
// region with (m + n + 4) * maxabs <= 30000, maxabs the largest magnitude
// among the substitution scores and the two gap scores (dir16_limit), has
// every H, E, F and their sums bounded there (a path of m + n steps).  A
// larger region whose borders still fit runs the checked form (CHECK below)
// and is redone on the 32-bit lanes of dp_warp_dir if a value leaves the
// range; the rest run on 32-bit lanes from the start.
//
// Decisions come from equalities on the packed values, not from predicates:
// min.u16x2(x ^ y, 1) is 1 in the halves where x != y.  Nibble of cell (i, j):
//   bit 0   H is not the diagonal (diagonal wins every tie)
//   bit 1   with bit 0: H is E (else F), under the tie policy's order of F and E
//   bit 2   E(i, j) was opened from H(i, j-1)
//   bit 3   F(i, j) was opened from H(i-1, j)
// A local alignment's floor needs no bit: the traceback carries the score of
// the cell it stands on and stops where H is 0, which is where the 32-bit
// form sets its zero code.  Layout: the nibbles of virtual lane v's R rows at
// column j in word dir16_warp_word(stripe, k, v, n), k = j - 1 + v: a lane
// stores its two virtual lanes' words as one 8-byte store, and its stores of
// 4 consecutive steps fill one 32-byte sector (a traceback along a lane reads
// a new sector every few moves).
//
// Borders need no special case in the loop.  The high half starts one column
// early, at column 0, from a column -1 of sentinels (H = NEG16) and the
// sentinel residue (score -128 against every row): the recurrence then gives
// column 0 itself (global: the vertical gap run down column 0; local: 0).
// The low half runs one column past n at the end; that column, like the rows
// past m, is computed from sentinel scores and reaches no cell of the region.
#pragma once
#include <cstdint>

#include "pg_dpdir.cuh"

namespace pg {

constexpr int NEG16 = -32000;
constexpr int SENT16 = NCODES;                 // residue code of column -1 and past n
constexpr int NC16 = NCODES + 1;
constexpr int PROF16_BYTES = 2 * NC16 * 32 * 8; // per warp: low and high halves' profiles
constexpr uint32_t ONE2 = 0x00010001u;

__device__ __forceinline__ uint32_t v16max(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("max.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t v16min(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("min.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t v16add(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("add.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
// 1 in each half where a != b, else 0
__device__ __forceinline__ uint32_t v16ne(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a ^ b), "r"(ONE2));
    return d;
}
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s)
{
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
    return d;
}
__host__ __device__ __forceinline__ uint32_t pk16(int lo, int hi)
{
    return ((uint32_t)lo & 0xffffu) | ((uint32_t)hi << 16);
}
// a border value of the 32-bit helpers (whose sentinel is NEG = -2^30) in 16 bits
__device__ __forceinline__ int c16(int x) { return x < NEG16 ? NEG16 : x; }
__device__ __forceinline__ int lo16(uint32_t x) { return (int)(int16_t)(x & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t x) { return (int)(int16_t)(x >> 16); }
__device__ __forceinline__ int half16(uint32_t x, int h) { return h ? hi16(x) : lo16(x); }

// largest m + n that runs on 16-bit lanes (0: none)
__host__ __forceinline__ int dir16_limit(int maxabs)
{
    if (maxabs < 1) maxabs = 1;
    if (maxabs > 100) return 0;
    return 30000 / maxabs - 4;
}

__host__ __device__ __forceinline__ int dir16_rows(int m, int cap)
{
    const int RMAX = cap < 1 ? 1 : (cap > 8 ? 8 : cap);
    const int stripes = m > 0 ? (m + 64 * RMAX - 1) / (64 * RMAX) : 1;
    const int r = (m + 64 * stripes - 1) / (64 * stripes);
    return r < 1 ? 1 : r;
}

// A stripe's wavefront steps, rounded up to whole 4-step tiles
__host__ __device__ __forceinline__ int dir16_steps(int n) { return (n + 63 + 3) & ~3; }

__host__ __device__ __forceinline__ uint64_t dir16_bytes(int m, int n, int R)
{
    if (m <= 0 || n <= 0) return 0;
    const uint64_t stripes = (uint64_t)((m + 64 * R - 1) / (64 * R));
    return stripes * (uint64_t)dir16_steps(n) * 256ull;
}

// Word (32-bit) index of virtual lane v (0..63) at wavefront step k of stripe s
// in a whole-warp region: tiles of 4 steps, each lane's 8-byte words (its two
// virtual lanes) of the 4 steps filling one 32-byte sector, so that a
// traceback walk along a lane reads a new sector every few moves
__host__ __device__ __forceinline__ uint64_t dir16_warp_word(int s, int k, int v, int n)
{
    return ((((uint64_t)s * (uint64_t)(dir16_steps(n) >> 2) + (uint64_t)(k >> 2)) * 32u +
             (uint64_t)(v >> 1)) * 4u + (uint64_t)(k & 3)) * 2u + (uint64_t)(v & 1);
}

// prmt selectors: row q of each half's word, sign-extended to 16 bits
__device__ __forceinline__ constexpr uint32_t sx_sel(int q)
{
    return (uint32_t)q | ((uint32_t)(q | 8) << 4) | ((uint32_t)(4 + q) << 8) |
           ((uint32_t)((4 + q) | 8) << 12);
}

// CHECK: the region is beyond the size that bounds every value inside int16
// (its borders still fit): the kernel tracks the least and the greatest H of
// each half (local: the greatest, which its best cell tracking keeps anyway)
// and reports sat when one left [-30000, 30000].  H moves by at most the
// largest score magnitude from a neighbour, so the first value to leave the
// range is still exact and no wrapped value goes unseen; the caller then
// redoes the region on 32-bit lanes.
constexpr int SAT16_DP = 30000;

template <int TIE, int R, bool LOCAL, bool CHECK = false>
__device__ DirOut dp_warp_dir16(const uint8_t *__restrict__ V, int m,
                                const uint8_t *__restrict__ Hs, int n,
                                const int *__restrict__ ssm, uint2 *__restrict__ prof,
                                int go, int ge, EdgeD *__restrict__ bnd, uint32_t *__restrict__ dir)
{
    static_assert(R >= 1 && R <= 8, "a direction word holds 8 rows");
    const int lane = threadIdx.x & 31;
    constexpr bool E_FIRST = (TIE & TIE_E_BEFORE_F) != 0;
    constexpr bool OPEN_FIRST = (TIE & TIE_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;
    const uint32_t go2 = pk16(go, go), ge2 = pk16(ge, ge);
    uint2 *profLo = prof, *profHi = prof + NC16 * 32;
    int bs = 0, bi = 0, bj = 0;
    DirOut res;
    res.have = 0; res.ei = 0; res.ej = 0; res.score = 0;
    uint32_t hmn = pk16(0, 0), hmx = pk16(0, 0), lmx = pk16(0, 0);   // CHECK: extremes of H
    for (int rb = 0, stripe = 0; rb < m; rb += 64 * R, ++stripe) {
        const int rows_here = min(64 * R, m - rb);
        const int v_last = (rows_here - 1) / R;
        const int t_last = v_last >> 1;
        const bool last_block = rb + rows_here >= m;
        const bool lane_on = lane <= t_last;
        const int hi_on = (2 * lane + 1 <= v_last) ? 1 : 0;
        const int i_base = rb + 2 * lane * R;           // row above the low half
        // score profile of this lane's 2R rows (pads and the sentinel: -128)
        __syncwarp();
        {
            int vc[2 * R];
#pragma unroll
            for (int r = 0; r < 2 * R; ++r) {
                const int i = i_base + r + 1;
                vc[r] = (lane_on && i <= m) ? (int)__ldg(V + i - 1) : -1;
            }
            for (int q = 0; q < NC16; ++q) {
                int c = q + lane;            // q + lane < 2 * NC16 + 6: up to two wraps
                if (c >= NC16) c -= NC16;
                if (c >= NC16) c -= NC16;
                uint32_t w[4] = {0x80808080u, 0x80808080u, 0x80808080u, 0x80808080u};
                if (c < NCODES) {
#pragma unroll
                    for (int r = 0; r < 2 * R; ++r) {
                        const int h = r / R, rr = r - h * R;
                        const uint32_t b = vc[r] >= 0 ? ((uint32_t)ssm[vc[r] * 32 + c] & 0xffu) : 0x80u;
                        const int wi = 2 * h + (rr >> 2), sh = 8 * (rr & 3);
                        w[wi] = (w[wi] & ~(0xffu << sh)) | (b << sh);
                    }
                }
                profLo[c * 32 + lane] = make_uint2(w[0], w[1]);
                profHi[c * 32 + lane] = make_uint2(w[2], w[3]);
            }
        }
        __syncwarp();
        // column 0 of the low half's rows, column -1 (sentinels) of the high half's
        uint32_t Hl[R], Al[R], Gl[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int h0 = dir_col0<LOCAL>(min(i_base + r + 1, m), go, ge, gmax).h;
            Hl[r] = pk16(h0, NEG16);
            Al[r] = pk16(NEG16 + ge, NEG16);
            Gl[r] = pk16(h0 + go, NEG16 + go);
        }
        const EdgeD e_up = dir_col0<LOCAL>(min(i_base, m), go, ge, gmax);
        const EdgeD e_lo = dir_col0<LOCAL>(min(i_base + R, m), go, ge, gmax);
        const EdgeD e_hi = dir_col0<LOCAL>(min(i_base + 2 * R, m), go, ge, gmax);
        uint32_t in_h = pk16(e_up.h, e_lo.h), in_a = pk16(c16(e_up.a), c16(e_lo.a));
        uint32_t out_h = pk16(e_lo.h, e_hi.h), out_a = pk16(c16(e_lo.a), c16(e_hi.a));
        const uint32_t in_sel = lane == 0 ? 0x5410u : 0x5432u;
        // residues: the low half's column at this step, the high half's (one behind)
        int hc_lo = SENT16;
        int hc_next = SENT16;
        {
            const int j1 = -2 * lane + 1;                // low half's column at step 0
            if (j1 >= 1 && j1 <= n) hc_next = (int)__ldg(Hs + j1 - 1);
        }
        uint2 *dtile = reinterpret_cast<uint2 *>(dir) +
                       (uint64_t)stripe * (uint64_t)(dir16_steps(n) >> 2) * 128u + lane * 4;
        // local form: a lane's words go out two steps at a time, 16 bytes (an
        // even step's word waits in wprev for the odd step after it; wk = its
        // step, -1: none).  uneven10m_sw 11.94 -> 11.66 s, sw100k 8.97 -> 8.94
        // ms; the global form measured slower that way (xdrop1m 40.1 -> 43.0 ms)
        uint2 wprev = make_uint2(0u, 0u);
        int wk = -1;
        uint32_t sbs = 0, sbs_seen = 0;
        int sbp0 = 0, sbp1 = 0;
        const int nsteps = n + v_last;
        // one wavefront step (a lambda, so that the local form's loop can be
        // unrolled by two without a second copy of the source)
        auto step = [&](const int k) {
            const uint32_t rh = __shfl_up_sync(FULL, out_h, 1);
            const uint32_t ra = __shfl_up_sync(FULL, out_a, 1);
            const uint32_t dgH = in_h;
            const int j = k - 2 * lane + 1;              // low half's column; high half: j - 1
            uint32_t th = rh, ta = ra;
            if (rb == 0) {
                // row 0 (lane 0 is at column j >= 1): computed by every lane and
                // selected, no branch on the lane
                const int b0 = LOCAL ? 0 : c16(go + (j - 1) * gmax);
                th = lane == 0 ? (uint32_t)b0 : rh;
                ta = lane == 0 ? (uint32_t)NEG16 : ra;
            } else if (lane == 0) {
                EdgeD e;
                if (j <= n) e = bnd[j];
                else { e.h = 0; e.a = NEG16; }
                th = (uint32_t)c16(e.h); ta = (uint32_t)c16(e.a);
            }
            in_h = prmt(th, out_h, in_sel);
            in_a = prmt(ta, out_a, in_sel);
            const int hc_hi = hc_lo;
            hc_lo = hc_next;
            {
                const int jn = j + 1;
                hc_next = (jn >= 1 && jn <= n) ? (int)__ldg(Hs + jn - 1) : SENT16;
            }
            if (lane_on && j >= 1 && j <= n + hi_on) {
                const uint2 pl = profLo[hc_lo * 32 + lane];
                const uint2 ph = profHi[hc_hi * 32 + lane];
                uint32_t cA = in_a, cG = v16add(in_h, go2);
                uint32_t dH = dgH;
                uint32_t W0 = 0, W1 = 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t s2 = prmt(r < 4 ? pl.x : pl.y, r < 4 ? ph.x : ph.y, sx_sel(r & 3));
                    const uint32_t E = v16max(Al[r], Gl[r]);
                    const uint32_t pe = OPEN_FIRST ? (v16ne(E, Gl[r]) ^ ONE2) : v16ne(E, Al[r]);
                    const uint32_t dg = v16add(dH, s2);
                    const uint32_t X = v16max(dg, E);
                    const uint32_t F = v16max(cA, cG);
                    const uint32_t pf = OPEN_FIRST ? (v16ne(F, cG) ^ ONE2) : v16ne(F, cA);
                    const uint32_t Hv = LOCAL ? __vimax_s16x2_relu(X, F) : v16max(X, F);
                    const uint32_t nd = v16ne(Hv, dg);
                    const uint32_t ne = E_FIRST ? (v16ne(Hv, E) ^ ONE2) : v16ne(Hv, F);
                    const uint32_t nib = nd + 2u * ne + 4u * pe + 8u * pf;
                    if (r < 4) W0 += nib << (4 * (r & 3));
                    else W1 += nib << (4 * (r & 3));
                    const uint32_t G = v16add(Hv, go2);
                    cA = v16add(F, ge2);
                    cG = G;
                    dH = Hl[r];
                    Hl[r] = Hv;
                    Al[r] = v16add(E, ge2);
                    Gl[r] = G;
                    if (LOCAL) sbs = v16max(sbs, Hv);
                    if (CHECK && !LOCAL) { hmn = v16min(hmn, Hv); hmx = v16max(hmx, Hv); }
                }
                const uint2 wd = make_uint2(prmt(W0, W1, 0x5410u), prmt(W0, W1, 0x7632u));
                if (!LOCAL) {
                    dtile[(uint64_t)(k >> 2) * 128u + (uint64_t)(k & 3)] = wd;
                } else if (k & 1) {
                    uint2 *dst = dtile + (uint64_t)(k >> 2) * 128u + (uint64_t)(k & 2);
                    if (wk >= 0) *reinterpret_cast<uint4 *>(dst) = make_uint4(wprev.x, wprev.y, wd.x, wd.y);
                    else dst[1] = wd;
                    wk = -1;
                } else {
                    wprev = wd;
                    wk = k;
                }
                out_h = Hl[R - 1];
                out_a = cA;
                if (!last_block && lane == t_last) {
                    const int h = v_last & 1;
                    const int jb = j - h;
                    if (jb >= 1 && jb <= n) {
                        EdgeD e;
                        e.h = half16(out_h, h);
                        e.a = half16(out_a, h);
                        bnd[jb] = e;
                    }
                }
                if (LOCAL && sbs != sbs_seen) {
                    // a new maximum in this column: its first row
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int s = half16(sbs, h);
                        if (s != half16(sbs_seen, h)) {
                            int rr = R - 1;
#pragma unroll
                            for (int r = R - 1; r >= 0; --r)
                                if (half16(Hl[r], h) == s) rr = r;
                            const int p = ((j - h) << 3) | rr;
                            if (h) sbp1 = p; else sbp0 = p;
                        }
                    }
                    sbs_seen = sbs;
                }
            } else if (LOCAL && wk >= 0) {
                dtile[(uint64_t)(wk >> 2) * 128u + (uint64_t)(wk & 3)] = wprev;
                wk = -1;
            }
        };
        if (LOCAL) {
            // two steps per iteration: the row registers swap roles instead of
            // being moved (sw100k 9.43 -> 9.15 ms; the global form unrolled measured
            // slower, xdrop1m alignment 40.9 -> 43.1 ms)
#pragma unroll 2
            for (int k = 0; k < nsteps; ++k) step(k);
        } else {
            for (int k = 0; k < nsteps; ++k) step(k);
        }
        if (LOCAL && wk >= 0) dtile[(uint64_t)(wk >> 2) * 128u + (uint64_t)(wk & 3)] = wprev;
        __syncwarp();
        if (CHECK && LOCAL) lmx = v16max(lmx, sbs);
        if (LOCAL) {
            // the low half's rows come before the high half's: a tie keeps the low
            // half, and against earlier stripes a tie goes to the smaller column
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int s = half16(sbs, h);
                const int sp = h ? sbp1 : sbp0;
                const int sj = sp >> 3;
                if (s > 0 && (s > bs || (s == bs && sj < bj))) {
                    bs = s; bj = sj; bi = i_base + h * R + (sp & 7) + 1;
                }
            }
        }
        if (!LOCAL && last_block) {
            const int rl = (rows_here - 1) % R;
            const int h = v_last & 1;
            int hs = 0;
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r == rl) hs = half16(Hl[r], h);
            res.score = __shfl_sync(FULL, hs, t_last);
        }
    }
    if (LOCAL) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int os = __shfl_xor_sync(FULL, bs, o);
            const int oi = __shfl_xor_sync(FULL, bi, o);
            const int oj = __shfl_xor_sync(FULL, bj, o);
            const bool take = os > bs || (os == bs && (oj < bj || (oj == bj && oi < bi)));
            if (take) { bs = os; bi = oi; bj = oj; }
        }
        res.score = bs;
        res.have = bs > 0;
        res.ei = bi; res.ej = bj;
    }
    if (CHECK) {
        const uint32_t mx = LOCAL ? lmx : hmx;
        const bool out = lo16(mx) > SAT16_DP || hi16(mx) > SAT16_DP ||
                         (!LOCAL && (lo16(hmn) < -SAT16_DP || hi16(hmn) < -SAT16_DP));
        res.sat = __any_sync(FULL, out) ? 1 : 0;
    }
    return res;
}

// ---------------------------------------------------------------- two regions per warp
// A region of at most 32 R rows whose values provably fit int16 runs on half a
// warp: lanes 0-15 take one region, lanes 16-31 another of the same R, each
// half a wavefront of 32 virtual lanes over a single stripe.  A wavefront
// spends a step per virtual lane filling and another draining; on half a warp
// those ramps are half as long, and the two regions share every instruction.
// Layout of a region: the nibbles of virtual lane v (0..31) at wavefront step
// k = j - 1 + v in word k * 32 + v, a half-warp's two virtual lanes per lane
// stored as one 8-byte word (128 contiguous bytes per half-warp and step).

// rows per lane of a region on half a warp (m <= 256)
__host__ __device__ __forceinline__ int dir16_pair_rows(int m) { return m > 32 ? (m + 31) / 32 : 1; }

// Layout of a half-warp region: tiles of 4 wavefront steps; in a tile, each
// lane's 8-byte words (its two virtual lanes) of the 4 steps make one 32-byte
// sector: uint2 ((k / 4) * 16 + lane) * 4 + k % 4.  A traceback walk along a
// lane then reads a new sector every few moves instead of at every move.
__host__ __device__ __forceinline__ uint64_t dir16_pair_bytes(int m, int n)
{
    if (m <= 0 || n <= 0) return 0;
    return (uint64_t)((n + 31 + 3) / 4) * 512ull;
}
__host__ __device__ __forceinline__ uint64_t dir16_pair_word(int k, int v)
{
    return ((uint64_t)((k >> 2) * 16 + (v >> 1)) * 4u + (uint64_t)(k & 3)) * 2u + (uint64_t)(v & 1);
}

// Each lane passes its half-warp's region (m = 0: none); R >= dir16_pair_rows(m)
// for both.  The result is that of the lane's own region.
template <int TIE, int R, bool LOCAL>
__device__ DirOut dp_pair_dir16(const uint8_t *__restrict__ V, int m,
                                const uint8_t *__restrict__ Hs, int n,
                                const int *__restrict__ ssm, uint2 *__restrict__ prof,
                                int go, int ge, uint32_t *__restrict__ dir)
{
    static_assert(R >= 1 && R <= 8, "a direction word holds 8 rows");
    const int lane = threadIdx.x & 31;
    const int sl = lane & 15;                     // lane within the half-warp
    constexpr bool E_FIRST = (TIE & TIE_E_BEFORE_F) != 0;
    constexpr bool OPEN_FIRST = (TIE & TIE_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;
    const uint32_t go2 = pk16(go, go), ge2 = pk16(ge, ge);
    uint2 *profLo = prof, *profHi = prof + NC16 * 32;
    const bool has = m > 0 && n > 0;
    const int v_last = has ? (m - 1) / R : -1;   // <= 31
    const int t_last = has ? v_last >> 1 : -1;
    const bool lane_on = sl <= t_last;
    const int hi_on = (2 * sl + 1 <= v_last) ? 1 : 0;
    const int i_base = 2 * sl * R;                // row above the low half
    __syncwarp();
    {
        int vc[2 * R];
#pragma unroll
        for (int r = 0; r < 2 * R; ++r) {
            const int i = i_base + r + 1;
            vc[r] = (lane_on && i <= m) ? (int)__ldg(V + i - 1) : -1;
        }
        for (int q = 0; q < NC16; ++q) {
            int c = q + lane;
            if (c >= NC16) c -= NC16;
            if (c >= NC16) c -= NC16;
            uint32_t w[4] = {0x80808080u, 0x80808080u, 0x80808080u, 0x80808080u};
            if (c < NCODES) {
#pragma unroll
                for (int r = 0; r < 2 * R; ++r) {
                    const int h = r / R, rr = r - h * R;
                    const uint32_t b = vc[r] >= 0 ? ((uint32_t)ssm[vc[r] * 32 + c] & 0xffu) : 0x80u;
                    const int wi = 2 * h + (rr >> 2), sh = 8 * (rr & 3);
                    w[wi] = (w[wi] & ~(0xffu << sh)) | (b << sh);
                }
            }
            profLo[c * 32 + lane] = make_uint2(w[0], w[1]);
            profHi[c * 32 + lane] = make_uint2(w[2], w[3]);
        }
    }
    __syncwarp();
    uint32_t Hl[R], Al[R], Gl[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int h0 = dir_col0<LOCAL>(min(i_base + r + 1, m), go, ge, gmax).h;
        Hl[r] = pk16(h0, NEG16);
        Al[r] = pk16(NEG16 + ge, NEG16);
        Gl[r] = pk16(h0 + go, NEG16 + go);
    }
    const EdgeD e_up = dir_col0<LOCAL>(min(i_base, m), go, ge, gmax);
    const EdgeD e_lo = dir_col0<LOCAL>(min(i_base + R, m), go, ge, gmax);
    const EdgeD e_hi = dir_col0<LOCAL>(min(i_base + 2 * R, m), go, ge, gmax);
    uint32_t in_h = pk16(e_up.h, e_lo.h), in_a = pk16(c16(e_up.a), c16(e_lo.a));
    uint32_t out_h = pk16(e_lo.h, e_hi.h), out_a = pk16(c16(e_lo.a), c16(e_hi.a));
    const uint32_t in_sel = sl == 0 ? 0x5410u : 0x5432u;
    int hc_lo = SENT16;
    int hc_next = SENT16;
    {
        const int j1 = -2 * sl + 1;
        if (j1 >= 1 && j1 <= n) hc_next = (int)__ldg(Hs + j1 - 1);
    }
    uint2 *dtile = reinterpret_cast<uint2 *>(dir) + sl * 4;
    // local form: a lane's words go out two steps at a time, as in dp_warp_dir16
    uint2 wprev = make_uint2(0u, 0u);
    int wk = -1;
    uint32_t sbs = 0, sbs_seen = 0;
    int sbp0 = 0, sbp1 = 0;
    int nsteps = has ? n + v_last : 0;
    nsteps = max(nsteps, __shfl_xor_sync(FULL, nsteps, 16));
    // one wavefront step (a lambda, so that the local form's loop can be
    // unrolled by two without a second copy of the source)
    auto step = [&](const int k) {
        const uint32_t rh = __shfl_up_sync(FULL, out_h, 1, 16);
        const uint32_t ra = __shfl_up_sync(FULL, out_a, 1, 16);
        const uint32_t dgH = in_h;
        const int j = k - 2 * sl + 1;
        // row 0 for the first lane of each half-warp, selected without a branch
        const int b0 = LOCAL ? 0 : c16(go + (j - 1) * gmax);
        const uint32_t th = sl == 0 ? (uint32_t)b0 : rh;
        const uint32_t ta = sl == 0 ? (uint32_t)NEG16 : ra;
        in_h = prmt(th, out_h, in_sel);
        in_a = prmt(ta, out_a, in_sel);
        const int hc_hi = hc_lo;
        hc_lo = hc_next;
        {
            const int jn = j + 1;
            hc_next = (jn >= 1 && jn <= n) ? (int)__ldg(Hs + jn - 1) : SENT16;
        }
        if (lane_on && j >= 1 && j <= n + hi_on) {
            const uint2 pl = profLo[hc_lo * 32 + lane];
            const uint2 ph = profHi[hc_hi * 32 + lane];
            uint32_t cA = in_a, cG = v16add(in_h, go2);
            uint32_t dH = dgH;
            uint32_t W0 = 0, W1 = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t s2 = prmt(r < 4 ? pl.x : pl.y, r < 4 ? ph.x : ph.y, sx_sel(r & 3));
                const uint32_t E = v16max(Al[r], Gl[r]);
                const uint32_t pe = OPEN_FIRST ? (v16ne(E, Gl[r]) ^ ONE2) : v16ne(E, Al[r]);
                const uint32_t dg = v16add(dH, s2);
                const uint32_t X = v16max(dg, E);
                const uint32_t F = v16max(cA, cG);
                const uint32_t pf = OPEN_FIRST ? (v16ne(F, cG) ^ ONE2) : v16ne(F, cA);
                const uint32_t Hv = LOCAL ? __vimax_s16x2_relu(X, F) : v16max(X, F);
                const uint32_t nd = v16ne(Hv, dg);
                const uint32_t ne = E_FIRST ? (v16ne(Hv, E) ^ ONE2) : v16ne(Hv, F);
                const uint32_t nib = nd + 2u * ne + 4u * pe + 8u * pf;
                if (r < 4) W0 += nib << (4 * (r & 3));
                else W1 += nib << (4 * (r & 3));
                const uint32_t G = v16add(Hv, go2);
                cA = v16add(F, ge2);
                cG = G;
                dH = Hl[r];
                Hl[r] = Hv;
                Al[r] = v16add(E, ge2);
                Gl[r] = G;
                if (LOCAL) sbs = v16max(sbs, Hv);
            }
            const uint2 wd = make_uint2(prmt(W0, W1, 0x5410u), prmt(W0, W1, 0x7632u));
            if (!LOCAL) {
                dtile[(uint64_t)(k >> 2) * 64u + (uint64_t)(k & 3)] = wd;
            } else if (k & 1) {
                uint2 *dst = dtile + (uint64_t)(k >> 2) * 64u + (uint64_t)(k & 2);
                if (wk >= 0) *reinterpret_cast<uint4 *>(dst) = make_uint4(wprev.x, wprev.y, wd.x, wd.y);
                else dst[1] = wd;
                wk = -1;
            } else {
                wprev = wd;
                wk = k;
            }
            out_h = Hl[R - 1];
            out_a = cA;
            if (LOCAL && sbs != sbs_seen) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int s = half16(sbs, h);
                    if (s != half16(sbs_seen, h)) {
                        int rr = R - 1;
#pragma unroll
                        for (int r = R - 1; r >= 0; --r)
                            if (half16(Hl[r], h) == s) rr = r;
                        const int p = ((j - h) << 3) | rr;
                        if (h) sbp1 = p; else sbp0 = p;
                    }
                }
                sbs_seen = sbs;
            }
        } else if (LOCAL && wk >= 0) {
            dtile[(uint64_t)(wk >> 2) * 64u + (uint64_t)(wk & 3)] = wprev;
            wk = -1;
        }
    };
    if (LOCAL) {
        // two steps per iteration: the row registers swap roles instead of
        // being moved (sw100k 9.43 -> 9.15 ms; the global form unrolled measured
        // slower, xdrop1m alignment 40.9 -> 43.1 ms)
#pragma unroll 2
        for (int k = 0; k < nsteps; ++k) step(k);
    } else {
        for (int k = 0; k < nsteps; ++k) step(k);
    }
    if (LOCAL && wk >= 0) dtile[(uint64_t)(wk >> 2) * 64u + (uint64_t)(wk & 3)] = wprev;
    __syncwarp();
    DirOut res;
    res.have = 0; res.ei = 0; res.ej = 0; res.score = 0;
    if (LOCAL) {
        // first maximum in column-major order: the low half's rows before the
        // high half's in a column, then the smaller column, then the smaller row
        int bs = 0, bi = 0, bj = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int s = half16(sbs, h);
            const int sp = h ? sbp1 : sbp0;
            const int sj = sp >> 3;
            if (s > 0 && (s > bs || (s == bs && sj < bj))) {
                bs = s; bj = sj; bi = i_base + h * R + (sp & 7) + 1;
            }
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            const int os = __shfl_xor_sync(FULL, bs, o);
            const int oi = __shfl_xor_sync(FULL, bi, o);
            const int oj = __shfl_xor_sync(FULL, bj, o);
            const bool take = os > bs || (os == bs && (oj < bj || (oj == bj && oi < bi)));
            if (take) { bs = os; bi = oi; bj = oj; }
        }
        res.score = bs;
        res.have = bs > 0;
        res.ei = bi; res.ej = bj;
    } else {
        const int rl = has ? (m - 1) % R : -1;
        const int h = v_last & 1;
        int hs = 0;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r == rl) hs = half16(Hl[r], h);
        res.score = __shfl_sync(FULL, hs, (lane & 16) + (t_last > 0 ? t_last : 0));
    }
    return res;
}

}  // namespace pg
