// pg_dp.cuh -- warp-level affine DP with traceback-equivalent statistics (sm_103a).
//
// One warp aligns one region.  Rows (V, the row sequence) are striped over the
// 32 lanes, R consecutive rows per lane; the warp sweeps the columns (H, the
// column sequence) as a wavefront: at step k lane t works on column k - t + 1
// and hands the values of its bottom row to lane t + 1 with __shfl_up_sync.
// Regions taller than 32*R rows are done in row blocks; the bottom row of each
// block goes through a per-warp scratch row (bnd) to the next block.
//
// Recurrence (the same as the oracle's, src/align/SeqanFullAligner.cpp:231 /
// SeqanXdropAligner.cpp:296 semantics):
//   E(i,j) = max(E(i,j-1) + ext, H(i,j-1) + first)      horizontal gap
//   F(i,j) = max(F(i-1,j) + ext, H(i-1,j) + first)      vertical gap
//   H(i,j) = max(H(i-1,j-1) + s, F, E [, 0])
// Statistics (M | D<<16, gap runs G, local begin) follow the predecessor a
// traceback would choose under the tie policy TIE, so the end cell carries the
// statistics computeAlignmentStats reports for the traced alignment.  A gap
// opened from a cell whose own best path already ends in a gap of the same
// orientation continues that run (G unchanged), as in the final alignment.
#pragma once
#include <cstdint>

namespace pg {

constexpr int NEG = -(1 << 30);
constexpr unsigned FULL = 0xffffffffu;

constexpr int TIE_E_BEFORE_F = 1;
constexpr int TIE_OPEN_FIRST = 2;

// statistics of the best path into a cell state
struct St {
    uint32_t md;  // matches | diagonal columns << 16
    uint32_t g;   // gap runs
    uint32_t b;   // local: first aligned residue, V index | H index << 16
};

__device__ __forceinline__ St st_sel(bool p, const St &a, const St &b)
{
    St r;
    r.md = p ? a.md : b.md;
    r.g = p ? a.g : b.g;
    r.b = p ? a.b : b.b;
    return r;
}
__device__ __forceinline__ St st_open(const St &a) { St r = a; r.g += 1; return r; }

// values a lane hands down (the bottom row of its stripe at one column)
struct Edge {
    int h, f;
    St sf, shof, sh;  // F stats, stats for a vertical open from H, H stats
};

template <bool LOCAL>
__device__ __forceinline__ Edge edge_shfl_up(const Edge &e)
{
    Edge r;
    r.h = __shfl_up_sync(FULL, e.h, 1);
    r.f = __shfl_up_sync(FULL, e.f, 1);
    r.sf.md = __shfl_up_sync(FULL, e.sf.md, 1);
    r.sf.g = __shfl_up_sync(FULL, e.sf.g, 1);
    r.shof.md = __shfl_up_sync(FULL, e.shof.md, 1);
    r.shof.g = __shfl_up_sync(FULL, e.shof.g, 1);
    r.sh.md = __shfl_up_sync(FULL, e.sh.md, 1);
    r.sh.g = __shfl_up_sync(FULL, e.sh.g, 1);
    if (LOCAL) {
        r.sf.b = __shfl_up_sync(FULL, e.sf.b, 1);
        r.shof.b = __shfl_up_sync(FULL, e.shof.b, 1);
        r.sh.b = __shfl_up_sync(FULL, e.sh.b, 1);
    } else {
        r.sf.b = r.shof.b = r.sh.b = 0;
    }
    return r;
}

// Column-0 / row-0 border cells (the recurrence restricted to one direction):
// global: H = first + (k-1) * max(first, ext), one gap run; local: 0, restart.
template <bool LOCAL>
__device__ __forceinline__ Edge border_row0(int j, int go, int gmax)
{
    Edge e;
    e.f = NEG;
    e.sf = St{0, 0, 0};
    if (LOCAL) {
        e.h = 0;
        e.sh = St{0, 0, (uint32_t)j << 16};
        e.shof = st_open(e.sh);
    } else if (j == 0) {
        e.h = 0;
        e.sh = St{0, 0, 0};
        e.shof = st_open(e.sh);
    } else {
        e.h = go + (j - 1) * gmax;
        e.sh = St{0, 1, 0};           // ends in a horizontal gap
        e.shof = st_open(e.sh);       // a vertical gap starts a new run
    }
    return e;
}

// row i of column 0, as the edge handed down from that row
template <bool LOCAL>
__device__ __forceinline__ Edge border_col0(int i, int go, int gmax)
{
    Edge e;
    if (LOCAL) {
        e.h = 0; e.f = NEG;
        e.sh = St{0, 0, (uint32_t)i};
        e.sf = St{0, 0, 0};
        e.shof = st_open(e.sh);
    } else if (i == 0) {
        e.h = 0; e.f = NEG;
        e.sh = St{0, 0, 0};
        e.sf = St{0, 0, 0};
        e.shof = st_open(e.sh);
    } else {
        e.h = go + (i - 1) * gmax;
        e.f = e.h;                     // column 0 is a vertical gap
        e.sh = St{0, 1, 0};
        e.sf = e.sh;
        e.shof = e.sh;                 // a further vertical gap continues the run
    }
    return e;
}

struct DpOut {
    int score;
    St st;
    int ei, ej;     // end cell (DP coordinates, local only)
    int have;       // local: a positive cell exists
};

// Align V[0,m) (rows) with Hs[0,n) (columns).  ssm: 32x32 int score table in
// shared memory indexed [v*32 + h].  bnd: per-warp scratch of n+1 Edge
// entries (used when m > 32*R).  All lanes return the same DpOut.
template <bool LOCAL, int TIE, int R>
__device__ DpOut dp_warp(const uint8_t *__restrict__ V, int m,
                         const uint8_t *__restrict__ Hs, int n,
                         const int *__restrict__ ssm, int go, int ge,
                         Edge *__restrict__ bnd)
{
    const int lane = threadIdx.x & 31;
    constexpr bool E_FIRST = (TIE & TIE_E_BEFORE_F) != 0;
    constexpr bool OPEN_FIRST = (TIE & TIE_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;

    // local best (score, then smaller j, then smaller i)
    int bs = 0, bi = 0, bj = 0;
    St bst{0, 0, 0};
    DpOut res;
    res.have = 0; res.ei = 0; res.ej = 0; res.score = 0; res.st = St{0, 0, 0};

    if (m == 0 || n == 0) {
        if (!LOCAL) {
            if (m == 0 && n == 0) { res.score = 0; }
            else { int k = m + n; res.score = go + (k - 1) * gmax; res.st = St{0, 1, 0}; }
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
        St SHl[R], SEl[R], SHoEl[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = rb + lane * R + r + 1;
            valid[r] = lane_on && i <= m;
            vrow[r] = valid[r] ? (int)__ldg(V + i - 1) * 32 : 0;
            Edge c0 = border_col0<LOCAL>(i, go, gmax);
            Hl[r] = c0.h;
            El[r] = NEG;
            SHl[r] = c0.sh;
            SEl[r] = St{0, 0, 0};
            // a horizontal gap opened from column 0 starts a new run
            SHoEl[r] = st_open(c0.sh);
        }
        const int i_up = rb + lane * R;
        int i_bot = rb + lane * R + R;
        if (i_bot > m) i_bot = m;
        Edge in = border_col0<LOCAL>(i_up, go, gmax);
        Edge out = border_col0<LOCAL>(i_bot, go, gmax);

        const int nsteps = n + t_last;
        for (int k = 0; k < nsteps; ++k) {
            Edge rcv = edge_shfl_up<LOCAL>(out);
            const int dgH = in.h;
            const St dgS = in.sh;
            if (lane == 0) {
                const int jn = k + 1;
                if (rb == 0) in = border_row0<LOCAL>(jn, go, gmax);
                else if (jn <= n) in = bnd[jn];
            } else {
                in = rcv;
            }
            const int j = k - lane + 1;
            if (lane_on && j >= 1 && j <= n) {
                const int hc = (int)__ldg(Hs + j - 1);
                int cH = in.h, cF = in.f;
                St cSF = in.sf, cSHoF = in.shof, cSH = in.sh;
                int dH = dgH;
                St dS = dgS;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!valid[r]) continue;
                    const int i = rb + lane * R + r + 1;
                    const int s = ssm[vrow[r] + hc];
                    // E (from the left)
                    bool pe;
                    int E;
                    {
                        const int ext = El[r] + ge, opn = Hl[r] + go;
                        if (OPEN_FIRST) { E = __vibmax_s32(opn, ext, &pe); }
                        else { bool px; E = __vibmax_s32(ext, opn, &px); pe = !px; }
                    }
                    const St SE = st_sel(pe, SHoEl[r], SEl[r]);
                    // F (from above)
                    bool pf;
                    int F;
                    {
                        const int ext = cF + ge, opn = cH + go;
                        if (OPEN_FIRST) { F = __vibmax_s32(opn, ext, &pf); }
                        else { bool px; F = __vibmax_s32(ext, opn, &px); pf = !px; }
                    }
                    const St SF = st_sel(pf, cSHoF, cSF);
                    // H
                    const int dg = dH + s;
                    St SD = dS;
                    SD.md += (1u << 16) + (uint32_t)((vrow[r] >> 5) == hc);
                    int Hv;
                    bool chE = false, chF = false;
                    St SH;
                    if (E_FIRST) {
                        bool p1, p2;
                        int t = __vibmax_s32(dg, E, &p1);
                        Hv = __vibmax_s32(t, F, &p2);
                        chE = !p1 && p2;
                        chF = !p2;
                        SH = st_sel(chF, SF, st_sel(chE, SE, SD));
                    } else {
                        bool p1, p2;
                        int t = __vibmax_s32(dg, F, &p1);
                        Hv = __vibmax_s32(t, E, &p2);
                        chF = !p1 && p2;
                        chE = !p2;
                        SH = st_sel(chE, SE, st_sel(chF, SF, SD));
                    }
                    if (LOCAL) {
                        if (Hv <= 0) {
                            Hv = 0;
                            chE = chF = false;
                            SH = St{0, 0, (uint32_t)i | ((uint32_t)j << 16)};
                        }
                    }
                    const St SHo = st_open(SH);
                    const St SHoE = chE ? SH : SHo;
                    const St SHoF = chF ? SH : SHo;
                    // the old left value is the diagonal of the next row
                    dH = Hl[r];
                    dS = SHl[r];
                    Hl[r] = Hv; El[r] = E; SEl[r] = SE; SHoEl[r] = SHoE; SHl[r] = SH;
                    cH = Hv; cF = F; cSF = SF; cSHoF = SHoF; cSH = SH;
                    if (LOCAL) {
                        // first maximum in column-major order; within a lane a
                        // later row block can only win a tie by a smaller column
                        if (Hv > bs || (Hv == bs && Hv > 0 && j < bj)) { bs = Hv; bi = i; bj = j; bst = SH; }
                    }
                }
                out.h = cH; out.f = cF; out.sf = cSF; out.shof = cSHoF; out.sh = cSH;
                if (!last_block && lane == t_last) bnd[j] = out;
            }
        }
        __syncwarp();
        if (!LOCAL && last_block) {
            // H(m, n) lives in lane t_last, row (rows_here - 1) % R
            const int rl = (rows_here - 1) % R;
            int hs = 0;
            St hst{0, 0, 0};
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r == rl) { hs = Hl[r]; hst = SHl[r]; }
            res.score = __shfl_sync(FULL, hs, t_last);
            res.st.md = __shfl_sync(FULL, hst.md, t_last);
            res.st.g = __shfl_sync(FULL, hst.g, t_last);
            res.st.b = 0;
        }
    }

    if (LOCAL) {
        // warp reduction: larger score, then smaller j, then smaller i
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            int os = __shfl_xor_sync(FULL, bs, o);
            int oi = __shfl_xor_sync(FULL, bi, o);
            int oj = __shfl_xor_sync(FULL, bj, o);
            uint32_t omd = __shfl_xor_sync(FULL, bst.md, o);
            uint32_t og = __shfl_xor_sync(FULL, bst.g, o);
            uint32_t ob = __shfl_xor_sync(FULL, bst.b, o);
            bool take = os > bs || (os == bs && (oj < bj || (oj == bj && oi < bi)));
            if (take) { bs = os; bi = oi; bj = oj; bst = St{omd, og, ob}; }
        }
        res.score = bs;
        res.have = bs > 0;
        res.ei = bi; res.ej = bj;
        res.st = bst;
    }
    return res;
}

// dispatch on the stripe height
template <bool LOCAL, int TIE>
__device__ __forceinline__ DpOut dp_dispatch(const uint8_t *V, int m, const uint8_t *Hs, int n,
                                             const int *ssm, int go, int ge, Edge *bnd)
{
    if (m <= 32) return dp_warp<LOCAL, TIE, 1>(V, m, Hs, n, ssm, go, ge, bnd);
    if (m <= 64) return dp_warp<LOCAL, TIE, 2>(V, m, Hs, n, ssm, go, ge, bnd);
    if (m <= 128) return dp_warp<LOCAL, TIE, 4>(V, m, Hs, n, ssm, go, ge, bnd);
    return dp_warp<LOCAL, TIE, 8>(V, m, Hs, n, ssm, go, ge, bnd);
}

}  // namespace pg
