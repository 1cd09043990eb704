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
// The maxima use the DPX __vibmax_s32, whose predicate gives the winner.
// Statistics (pg_stats.cuh) follow the predecessor a traceback would choose
// under the tie policy TIE, so the end cell carries the statistics of the
// traced alignment.  A gap opened from a cell whose best path already ends in
// a gap of the same orientation continues that run (G unchanged), as in the
// final alignment.
#pragma once
#include <cstdint>

#include "pg_stats.cuh"

namespace pg {

constexpr int NEG = -(1 << 30);
constexpr unsigned FULL = 0xffffffffu;

constexpr int TIE_E_BEFORE_F = 1;
constexpr int TIE_OPEN_FIRST = 2;

// values a lane hands down (the bottom row of its stripe at one column)
template <class S>
struct Edge {
    int h, f;
    S sf, shof, sh;  // F stats, stats for a vertical open from H, H stats
    __device__ __forceinline__ Edge shfl_up() const
    {
        Edge r;
        r.h = __shfl_up_sync(FULL, h, 1);
        r.f = __shfl_up_sync(FULL, f, 1);
        r.sf = sf.shfl_up();
        r.shof = shof.shfl_up();
        r.sh = sh.shfl_up();
        return r;
    }
};

// Row 0 / column 0: the recurrence restricted to one direction.  Global: H =
// first + (k-1) * max(first, ext), one gap run.  Local: 0, alignment restarts.
template <class S>
__device__ __forceinline__ Edge<S> border_row0(int j, int go, int gmax)
{
    Edge<S> e;
    e.f = NEG;
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
__device__ __forceinline__ Edge<S> border_col0(int i, int go, int gmax)
{
    Edge<S> e;
    if (S::LOCAL) {
        e.h = 0; e.f = NEG;
        e.sh = S::reset(i, 0);
        e.sf = S::zero();
        e.shof = e.sh.open();
    } else if (i == 0) {
        e.h = 0; e.f = NEG;
        e.sh = S::zero();
        e.sf = S::zero();
        e.shof = e.sh.open();
    } else {
        e.h = go + (i - 1) * gmax;
        e.f = e.h;                   // column 0 is a vertical gap
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
// shared memory indexed [v*32 + h].  bnd: per-warp scratch of n+1 edges (used
// when m > 32*R).  All lanes return the same DpOut.
template <class S, int TIE, int R>
__device__ DpOut<S> dp_warp(const uint8_t *__restrict__ V, int m,
                            const uint8_t *__restrict__ Hs, int n,
                            const int *__restrict__ ssm, int go, int ge,
                            Edge<S> *__restrict__ bnd)
{
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

        int vrow[R];
        bool valid[R];
        int Hl[R], El[R];
        S SHl[R], SEl[R], SHoEl[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = rb + lane * R + r + 1;
            valid[r] = lane_on && i <= m;
            vrow[r] = valid[r] ? (int)__ldg(V + i - 1) * 32 : 0;
            const Edge<S> c0 = border_col0<S>(i, go, gmax);
            Hl[r] = c0.h;
            El[r] = NEG;
            SHl[r] = c0.sh;
            SEl[r] = S::zero();
            SHoEl[r] = c0.sh.open();   // a horizontal gap from column 0 starts a run
        }
        const int i_up = rb + lane * R;
        const int i_bot = min(rb + lane * R + R, m);
        Edge<S> in = border_col0<S>(i_up, go, gmax);
        Edge<S> out = border_col0<S>(i_bot, go, gmax);

        const int nsteps = n + t_last;
        for (int k = 0; k < nsteps; ++k) {
            const Edge<S> rcv = out.shfl_up();
            const int dgH = in.h;
            const S dgS = in.sh;
            if (lane == 0) {
                const int jn = k + 1;
                if (rb == 0) in = border_row0<S>(jn, go, gmax);
                else if (jn <= n) in = bnd[jn];
            } else {
                in = rcv;
            }
            const int j = k - lane + 1;
            if (lane_on && j >= 1 && j <= n) {
                const int hc = (int)__ldg(Hs + j - 1);
                int cH = in.h, cF = in.f;
                S cSF = in.sf, cSHoF = in.shof, cSH = in.sh;
                int dH = dgH;
                S dS = dgS;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!valid[r]) continue;
                    const int s = ssm[vrow[r] + hc];
                    // E (from the left)
                    bool pe;
                    int E;
                    if (OPEN_FIRST) { E = __vibmax_s32(Hl[r] + go, El[r] + ge, &pe); }
                    else { bool px; E = __vibmax_s32(El[r] + ge, Hl[r] + go, &px); pe = !px; }
                    const S SE = S::sel(pe, SHoEl[r], SEl[r]);
                    // F (from above)
                    bool pf;
                    int F;
                    if (OPEN_FIRST) { F = __vibmax_s32(cH + go, cF + ge, &pf); }
                    else { bool px; F = __vibmax_s32(cF + ge, cH + go, &px); pf = !px; }
                    const S SF = S::sel(pf, cSHoF, cSF);
                    // H
                    const int dg = dH + s;
                    const S SD = dS.diag((uint32_t)((vrow[r] >> 5) == hc));
                    int Hv;
                    bool chE, chF;
                    S SH;
                    if (E_FIRST) {
                        bool p1, p2;
                        const int t = __vibmax_s32(dg, E, &p1);
                        Hv = __vibmax_s32(t, F, &p2);
                        chF = !p2;
                        chE = p2 && !p1;
                        SH = S::sel(chF, SF, S::sel(chE, SE, SD));
                    } else {
                        bool p1, p2;
                        const int t = __vibmax_s32(dg, F, &p1);
                        Hv = __vibmax_s32(t, E, &p2);
                        chE = !p2;
                        chF = p2 && !p1;
                        SH = S::sel(chE, SE, S::sel(chF, SF, SD));
                    }
                    if (S::LOCAL) {
                        if (Hv <= 0) {
                            Hv = 0;
                            chE = chF = false;
                            SH = S::reset(rb + lane * R + r + 1, j);
                        }
                    }
                    const S SHo = SH.open();
                    const S SHoE = S::sel(chE, SH, SHo);
                    const S SHoF = S::sel(chF, SH, SHo);
                    // the old left value is the diagonal of the next row
                    dH = Hl[r];
                    dS = SHl[r];
                    Hl[r] = Hv; El[r] = E; SEl[r] = SE; SHoEl[r] = SHoE; SHl[r] = SH;
                    cH = Hv; cF = F; cSF = SF; cSHoF = SHoF; cSH = SH;
                    if (S::LOCAL) {
                        // first maximum in column-major order; within a lane a
                        // later row block can only win a tie by a smaller column
                        if (Hv > bs || (Hv == bs && Hv > 0 && j < bj)) {
                            bs = Hv; bi = rb + lane * R + r + 1; bj = j; bst = SH;
                        }
                    }
                }
                out.h = cH; out.f = cF; out.sf = cSF; out.shof = cSHoF; out.sh = cSH;
                if (!last_block && lane == t_last) bnd[j] = out;
            }
        }
        __syncwarp();
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
