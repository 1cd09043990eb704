// pg_dp.cuh -- warp-level affine DP with traceback-equivalent statistics (sm_103a).
//
// One warp aligns one region.  Rows (V, the row sequence) are striped over the
// 32 lanes, R consecutive rows per lane; the warp sweeps the columns (H, the
// column sequence) as a wavefront: at step k lane t works on column k - t + 1
// and hands the values of its bottom row to lane t + 1 with __shfl_up_sync.
// Regions taller than 32*R rows are done in row blocks; the bottom row of each
// block goes through a per-warp scratch row (bnd) to the next block.
//
// Recurrence (the oracle's, i.e. the semantics of src/align/SeqanFullAligner.cpp:231
// and SeqanXdropAligner.cpp:296):
//   E(i,j) = max(E(i,j-1) + ext, H(i,j-1) + first)      horizontal gap
//   F(i,j) = max(F(i-1,j) + ext, H(i-1,j) + first)      vertical gap
//   H(i,j) = max(H(i-1,j-1) + s, F, E [, 0])
// Inside a lane only F runs down the rows.  The lane carries A = F + ext and
// G = H + first, so the chain from one row to the next is
//   F = vibmax(G_up, A_up)        H = max(X, F)        G = H + first
// with X = max(diag, E); the diagonal, E and every statistic select depend
// only on the previous column and sit off that chain.  (G as
// viaddmax(F, first, X + first) gives a two-op chain but one instruction more
// per cell; with the ALU pipe the bound, the shorter issue count measured
// 1-2 % faster.)  The DPX predicates give the winner of each
// maximum; statistics (pg_stats.cuh) follow the predecessor a traceback would
// choose under the tie policy TIE, so the end cell carries the statistics of
// the traced alignment.  A gap opened from a cell whose best path already ends
// in a gap of the same orientation continues that run (G unchanged), as in the
// final alignment.
//
// Substitution scores come from a per-lane profile in shared memory: for each
// residue code c, prof[c * 32 + lane] packs the scores of the lane's R rows
// against c as int8 (rows 0-3 in .x, 4-7 in .y).  One 64-bit load per column
// and lane, no bank conflicts, and a sign-extending byte extract per cell.
#pragma once
#include <cstdint>

#include "pg_stats.cuh"

namespace pg {

constexpr int NEG = -(1 << 30);
constexpr unsigned FULL = 0xffffffffu;
constexpr int NCODES = 25;              // residue codes
constexpr int PROF_BYTES = NCODES * 32 * 8;  // per-warp score profile

constexpr int TIE_E_BEFORE_F = 1;
constexpr int TIE_OPEN_FIRST = 2;

// values a lane hands down (the bottom row of its stripe at one column)
template <class S>
struct Edge {
    int h, a;        // H, and F + ext
    S sf, shof, sh;  // F stats, stats for a vertical open from H, H stats
    __device__ __forceinline__ Edge shfl_up() const
    {
        Edge r;
        r.h = __shfl_up_sync(FULL, h, 1);
        r.a = __shfl_up_sync(FULL, a, 1);
        r.sf = sf.shfl_up();
        r.shof = shof.shfl_up();
        r.sh = sh.shfl_up();
        return r;
    }
};

// Row 0 / column 0: the recurrence restricted to one direction.  Global: H =
// first + (k-1) * max(first, ext), one gap run.  Local: 0, alignment restarts.
template <class S>
__device__ __forceinline__ Edge<S> border_row0(int j, int go, int ge, int gmax)
{
    Edge<S> e;
    e.a = NEG + ge;
    e.sf = S::zero();
    if (S::LOCAL) {
        e.h = 0;
        e.sh = S::reset(0, j);
        e.shof = e.sh.open();
    } else if (j == 0) {
        e.h = 0;
        e.sh = S::zero();
        e.shof = e.sh.open();
    } else {
        e.h = go + (j - 1) * gmax;
        e.sh = S::gap1();           // ends in a horizontal gap
        e.shof = e.sh.open();       // a vertical gap starts a new run
    }
    return e;
}

template <class S>
__device__ __forceinline__ Edge<S> border_col0(int i, int go, int ge, int gmax)
{
    Edge<S> e;
    if (S::LOCAL) {
        e.h = 0; e.a = NEG + ge;
        e.sh = S::reset(i, 0);
        e.sf = S::zero();
        e.shof = e.sh.open();
    } else if (i == 0) {
        e.h = 0; e.a = NEG + ge;
        e.sh = S::zero();
        e.sf = S::zero();
        e.shof = e.sh.open();
    } else {
        e.h = go + (i - 1) * gmax;
        e.a = e.h + ge;              // column 0 is a vertical gap: F = H
        e.sh = S::gap1();
        e.sf = e.sh;
        e.shof = e.sh;               // a further vertical gap continues the run
    }
    return e;
}

template <class S>
struct DpOut {
    int score;
    S st;
    int ei, ej;     // end cell (DP coordinates, local only)
    int have;       // local: a positive cell exists
};

// Align V[0,m) (rows) with Hs[0,n) (columns).  ssm: 32x32 int score table in
// shared memory indexed [v*32 + h]; prof: this warp's profile buffer
// (PROF_BYTES); bnd: per-warp scratch of n+1 edges (used when m > 32*R).  All
// lanes return the same DpOut.
template <class S, int TIE, int R>
__device__ DpOut<S> dp_warp(const uint8_t *__restrict__ V, int m,
                            const uint8_t *__restrict__ Hs, int n,
                            const int *__restrict__ ssm, uint2 *__restrict__ prof,
                            int go, int ge, Edge<S> *__restrict__ bnd)
{
    static_assert(R >= 1 && R <= 8, "profile holds up to 8 rows per lane");
    const int lane = threadIdx.x & 31;
    constexpr bool E_FIRST = (TIE & TIE_E_BEFORE_F) != 0;
    constexpr bool OPEN_FIRST = (TIE & TIE_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;

    int bs = 0, bi = 0, bj = 0;  // local best: score, then smaller j, then smaller i
    S bst = S::zero();
    DpOut<S> res;
    res.have = 0; res.ei = 0; res.ej = 0; res.score = 0; res.st = S::zero();

    if (m == 0 || n == 0) {
        if (!S::LOCAL && (m + n) > 0) {
            res.score = go + (m + n - 1) * gmax;
            res.st = S::gap1();
        }
        return res;
    }

    for (int rb = 0; rb < m; rb += 32 * R) {
        const int rows_here = min(32 * R, m - rb);
        const int t_last = (rows_here - 1) / R;
        const bool last_block = rb + rows_here >= m;
        const bool lane_on = lane <= t_last;

        int vcode[R];
        bool valid[R];
        int Hl[R], Gl[R], Al[R];
        S SHl[R], SEl[R], SHoEl[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = rb + lane * R + r + 1;
            valid[r] = lane_on && i <= m;
            vcode[r] = valid[r] ? (int)__ldg(V + i - 1) : 255;
            const Edge<S> c0 = border_col0<S>(i, go, ge, gmax);
            Hl[r] = c0.h;
            Gl[r] = c0.h + go;
            Al[r] = NEG + ge;          // no horizontal gap ends in column 0
            SHl[r] = c0.sh;
            SEl[r] = S::zero();
            SHoEl[r] = c0.sh.open();   // a horizontal gap from column 0 starts a run
        }
        // this lane's score profile; lanes start at different residues so the
        // table reads spread over banks
        __syncwarp();
        for (int q = 0; q < NCODES; ++q) {
            int c = q + lane;
            if (c >= NCODES) c -= NCODES;
            if (c >= NCODES) c -= NCODES;
            uint32_t lo = 0, hi = 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t b = valid[r] ? ((uint32_t)ssm[vcode[r] * 32 + c] & 0xffu) : 0u;
                if (r < 4) lo |= b << (8 * r);
                else hi |= b << (8 * (r - 4));
            }
            prof[c * 32 + lane] = make_uint2(lo, hi);
        }
        __syncwarp();

        const int i_up = rb + lane * R;
        const int i_bot = min(rb + lane * R + R, m);
        Edge<S> in = border_col0<S>(i_up, go, ge, gmax);
        Edge<S> out = border_col0<S>(i_bot, go, ge, gmax);
        // residue of the column this lane works on next (prefetched one step ahead)
        int hc_next = (lane == 0) ? (int)__ldg(Hs) : 0;

        // this lane's first maximum in this row block: score, j << 3 | row, statistics
        int sbs = 0, sbp = 0;
        S sbst = S::zero();
        const int nsteps = n + t_last;
        // Two columns per trip for the local form lets the compiler alternate
        // register sets instead of copying the carried values (sw100k 352 ->
        // 376 GCUPS); the global form measured 15 % slower that way.
#pragma unroll (S::LOCAL ? 2 : 1)
        for (int k = 0; k < nsteps; ++k) {
            const Edge<S> rcv = out.shfl_up();
            const int dgH = in.h;
            const S dgS = in.sh;
            if (lane == 0) {
                const int jn = k + 1;
                if (rb == 0) in = border_row0<S>(jn, go, ge, gmax);
                else if (jn <= n) in = bnd[jn];
            } else {
                in = rcv;
            }
            const int j = k - lane + 1;
            const int hc = hc_next;
            hc_next = (j >= 0 && j < n) ? (int)__ldg(Hs + j) : 0;
            if (lane_on && j >= 1 && j <= n) {
                const int j8 = j << 3;
                const uint2 pw = prof[hc * 32 + lane];
                int cG = in.h + go, cA = in.a, cH = in.h;
                S cSF = in.sf, cSHoF = in.shof, cSH = in.sh;
                int dH = dgH;
                S dS = dgS;
                // Rows past m exist only at the end of the last lane's stripe:
                // they are computed (no branch) but feed nothing downstream --
                // the next lane is idle and the result is read from the last
                // valid row -- and they never enter the local best.
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int s = (int)(signed char)((r < 4 ? pw.x : pw.y) >> (8 * (r & 3)));
                    // ---- off the row chain: E, diagonal, their maximum X
                    bool pe;
                    int E;
                    if (OPEN_FIRST) { E = __vibmax_s32(Gl[r], Al[r], &pe); }
                    else { bool px; E = __vibmax_s32(Al[r], Gl[r], &px); pe = !px; }
                    const S SE = S::sel(pe, SHoEl[r], SEl[r]);
                    const int dg = dH + s;
                    const S SD = dS.diag((uint32_t)(vcode[r] == hc));
                    bool pX;                      // diagonal wins a tie with E
                    int X = __vibmax_s32(dg, E, &pX);
                    if (S::LOCAL) X = max(X, 0);
                    const S SX = S::sel(pX, SD, SE);
                    const S SXo = SX.open();
                    // ---- the row chain
                    bool pf;
                    int F;
                    if (OPEN_FIRST) { F = __vibmax_s32(cG, cA, &pf); }
                    else { bool px; F = __vibmax_s32(cA, cG, &px); pf = !px; }
                    const int A = F + ge;
                    // ---- H and its statistics
                    const int Hv = max(X, F);
                    const int G = Hv + go;
                    const bool chF = E_FIRST ? (F > X) : (F > dg && F >= E);
                    const S SF = S::sel(pf, cSHoF, cSF);
                    S SH = S::sel(chF, SF, SX);
                    S SHoF = S::sel(chF, SF, SXo);
                    bool chE = !pX && !chF;
                    if (S::LOCAL) {
                        if (Hv == 0) {
                            SH = S::reset(rb + lane * R + r + 1, j);
                            SHoF = SH.open();
                            chE = false;
                        }
                    }
                    const S SHoE = S::sel(chE, SH, SH.open());
                    // the old left value is the diagonal of the next row
                    dH = Hl[r];
                    dS = SHl[r];
                    Hl[r] = Hv; Gl[r] = G; Al[r] = E + ge;
                    SEl[r] = SE; SHoEl[r] = SHoE; SHl[r] = SH;
                    cG = G; cA = A; cH = Hv; cSF = SF; cSHoF = SHoF; cSH = SH;
                    if (S::LOCAL) {
                        // a lane meets its cells of one row block in column-major
                        // order, so the first maximum is a strict improvement
                        const bool take = valid[r] && Hv > sbs;
                        sbs = take ? Hv : sbs;
                        sbp = take ? j8 + r : sbp;
                        sbst = S::sel(take, SH, sbst);
                    }
                }
                out.h = cH; out.a = cA; out.sf = cSF; out.shof = cSHoF; out.sh = cSH;
                if (!last_block && lane == t_last) bnd[j] = out;
            }
        }
        __syncwarp();
        if (S::LOCAL && sbs > 0) {
            // first maximum in column-major order: against earlier row blocks
            // (smaller rows) a tie goes to the smaller column only
            const int sj = sbp >> 3;
            if (sbs > bs || (sbs == bs && sj < bj)) {
                bs = sbs; bj = sj; bi = rb + lane * R + (sbp & 7) + 1; bst = sbst;
            }
        }
        if (!S::LOCAL && last_block) {
            // H(m, n) lives in lane t_last, row (rows_here - 1) % R
            const int rl = (rows_here - 1) % R;
            int hs = 0;
            S hst = S::zero();
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r == rl) { hs = Hl[r]; hst = SHl[r]; }
            res.score = __shfl_sync(FULL, hs, t_last);
            res.st = hst.shfl(t_last);
        }
    }

    if (S::LOCAL) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int os = __shfl_xor_sync(FULL, bs, o);
            const int oi = __shfl_xor_sync(FULL, bi, o);
            const int oj = __shfl_xor_sync(FULL, bj, o);
            const S ost = bst.shfl_xor(o);
            const bool take = os > bs || (os == bs && (oj < bj || (oj == bj && oi < bi)));
            if (take) { bs = os; bi = oi; bj = oj; bst = ost; }
        }
        res.score = bs;
        res.have = bs > 0;
        res.ei = bi; res.ej = bj;
        res.st = bst;
    }
    return res;
}

}  // namespace pg
