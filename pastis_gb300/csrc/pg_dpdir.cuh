// pg_dpdir.cuh -- the alignment DP in traceback form (sm_103a).
//
// Same recurrence, borders, tie policy and warp-striped layout as dp_warp
// (pg_dp.cuh), but no statistics ride along: each cell stores the four
// decisions a traceback needs as one nibble, and a separate traceback pass
// (pg_trace.cuh) walks them back and counts matches, columns and gap runs.
// Per cell this drops the statistics words and their selects (most of
// dp_warp's instructions) for a nibble insert and half a byte of HBM write;
// the direction matrices of a whole batch sit in HBM between the two passes.
//
// Nibble of cell (i, j):
//   bits 0-1  where H came from: 0 diagonal, 1 F (vertical gap), 2 E
//             (horizontal gap), 3 the local floor (H = 0: the alignment starts
//             after this cell)
//   bit 2     E(i, j) was opened from H(i, j-1) (else extended from E(i, j-1))
//   bit 3     F(i, j) was opened from H(i-1, j) (else extended from F(i-1, j))
// Layout of one region: the nibbles of a lane's R rows at column j (row r of
// the lane in bits 4r..4r+3) sit in word (stripe * (n + 31) + k) * 32 + lane,
// k = j - 1 + lane the wavefront step that computes them, so every store of
// a warp fills 128 contiguous bytes (a [column][lane] layout scatters one
// step's 32 words over 32 lines: measured 2x the DRAM writes plus
// write-allocate reads), and a traceback moving left or up walks back through
// neighbouring lines.
#pragma once
#include <cstdint>

#include "pg_dp.cuh"

namespace pg {

constexpr uint32_t DIR_DIAG = 0, DIR_F = 1, DIR_E = 2, DIR_ZERO = 3;
constexpr uint32_t DIR_EOPEN = 4, DIR_FOPEN = 8;

// stripe-boundary edge without statistics
struct EdgeD {
    int h, a;   // H, and F + ext
    __device__ __forceinline__ EdgeD shfl_up() const
    {
        EdgeD r;
        r.h = __shfl_up_sync(FULL, h, 1);
        r.a = __shfl_up_sync(FULL, a, 1);
        return r;
    }
};

template <bool LOCAL>
__device__ __forceinline__ EdgeD dir_row0(int j, int go, int ge, int gmax)
{
    EdgeD e;
    e.a = NEG + ge;
    e.h = LOCAL ? 0 : (j == 0 ? 0 : go + (j - 1) * gmax);
    return e;
}

template <bool LOCAL>
__device__ __forceinline__ EdgeD dir_col0(int i, int go, int ge, int gmax)
{
    EdgeD e;
    if (LOCAL || i == 0) { e.h = 0; e.a = NEG + ge; }
    else { e.h = go + (i - 1) * gmax; e.a = e.h + ge; }
    return e;
}

// bytes of the direction matrix of an m x n region at R rows per lane
__host__ __device__ __forceinline__ uint64_t dir_bytes(int m, int n, int R)
{
    if (m <= 0 || n <= 0) return 0;
    const uint64_t stripes = (uint64_t)((m + 32 * R - 1) / (32 * R));
    return stripes * (uint64_t)(n + 31) * 128ull;
}

struct DirOut {
    int score;
    int ei, ej;     // local: first maximum in column-major order
    int have;
    int sat = 0;    // 16-bit lanes, checked form: a value left [-30000, 30000]
};

template <int TIE, int R, bool LOCAL>
__device__ DirOut dp_warp_dir(const uint8_t *__restrict__ V, int m,
                              const uint8_t *__restrict__ Hs, int n,
                              const int *__restrict__ ssm, uint2 *__restrict__ prof,
                              int go, int ge, EdgeD *__restrict__ bnd, uint32_t *__restrict__ dir)
{
    static_assert(R >= 1 && R <= 8, "a direction word holds 8 rows");
    const int lane = threadIdx.x & 31;
    constexpr bool E_FIRST = (TIE & TIE_E_BEFORE_F) != 0;
    constexpr bool OPEN_FIRST = (TIE & TIE_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;
    int bs = 0, bi = 0, bj = 0;
    DirOut res;
    res.have = 0; res.ei = 0; res.ej = 0; res.score = 0;
    for (int rb = 0, stripe = 0; rb < m; rb += 32 * R, ++stripe) {
        const int rows_here = min(32 * R, m - rb);
        const int t_last = (rows_here - 1) / R;
        const bool last_block = rb + rows_here >= m;
        const bool lane_on = lane <= t_last;
        int vcode[R];
        bool valid[R];
        int Hl[R], Al[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = rb + lane * R + r + 1;
            valid[r] = lane_on && i <= m;
            vcode[r] = valid[r] ? (int)__ldg(V + i - 1) : 255;
            Hl[r] = dir_col0<LOCAL>(i, go, ge, gmax).h;
            Al[r] = NEG + ge;
        }
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
        EdgeD in = dir_col0<LOCAL>(i_up, go, ge, gmax);
        EdgeD out = dir_col0<LOCAL>(i_bot, go, ge, gmax);
        int hc_next = (lane == 0) ? (int)__ldg(Hs) : 0;
        uint32_t *dstep = dir + (uint64_t)stripe * (uint64_t)(n + 31) * 32u + lane;
        int sbs = 0, sbp = 0;
        const int nsteps = n + t_last;
        for (int k = 0; k < nsteps; ++k) {
            const EdgeD rcv = out.shfl_up();
            const int dgH = in.h;
            if (lane == 0) {
                const int jn = k + 1;
                if (rb == 0) in = dir_row0<LOCAL>(jn, go, ge, gmax);
                else if (jn <= n) in = bnd[jn];
            } else {
                in = rcv;
            }
            const int j = k - lane + 1;
            const int hc = hc_next;
            hc_next = (j >= 0 && j < n) ? (int)__ldg(Hs + j) : 0;
            if (lane_on && j >= 1 && j <= n) {
                const uint2 pw = prof[hc * 32 + lane];
                int cG = in.h + go, cA = in.a, cH = in.h;
                int dH = dgH;
                uint32_t word = 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int s = (int)(signed char)((r < 4 ? pw.x : pw.y) >> (8 * (r & 3)));
                    bool pe;
                    int E;
                    if (OPEN_FIRST) { E = __vibmax_s32(Hl[r] + go, Al[r], &pe); }
                    else { bool px; E = __vibmax_s32(Al[r], Hl[r] + go, &px); pe = !px; }
                    const int dg = dH + s;
                    bool pX;
                    int X = __vibmax_s32(dg, E, &pX);
                    bool pf;
                    int F;
                    if (OPEN_FIRST) { F = __vibmax_s32(cG, cA, &pf); }
                    else { bool px; F = __vibmax_s32(cA, cG, &px); pf = !px; }
                    const int A = F + ge;
                    if (LOCAL) X = max(X, 0);
                    const int Hv = max(X, F);
                    const bool chF = E_FIRST ? (F > X) : (F > dg && F >= E);
                    uint32_t hsrc = chF ? DIR_F : (pX ? DIR_DIAG : DIR_E);
                    if (LOCAL && Hv == 0) hsrc = DIR_ZERO;
                    const uint32_t nib = hsrc | (pe ? DIR_EOPEN : 0u) | (pf ? DIR_FOPEN : 0u);
                    word |= nib << (4 * r);
                    dH = Hl[r];
                    Hl[r] = Hv;
                    Al[r] = E + ge;
                    cG = Hv + go; cA = A; cH = Hv;
                    if (LOCAL) {
                        const bool take = valid[r] && Hv > sbs;
                        sbs = take ? Hv : sbs;
                        sbp = take ? (j << 3) + r : sbp;
                    }
                }
                dstep[(uint64_t)k * 32u] = word;
                out.h = cH; out.a = cA;
                if (!last_block && lane == t_last) bnd[j] = out;
            }
        }
        __syncwarp();
        if (LOCAL && sbs > 0) {
            const int sj = sbp >> 3;
            if (sbs > bs || (sbs == bs && sj < bj)) { bs = sbs; bj = sj; bi = rb + lane * R + (sbp & 7) + 1; }
        }
        if (!LOCAL && last_block) {
            const int rl = (rows_here - 1) % R;
            int hs = 0;
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r == rl) hs = Hl[r];
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
    return res;
}

}  // namespace pg
