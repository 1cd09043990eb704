// pg_trace.cuh -- traceback over the direction nibbles of dp_warp_dir
// (pg_dpdir.cuh): one thread walks one region from its end cell back to its
// start and counts what computeAlignmentStats counts
// (src/align/SeqanFullAligner.cpp:238-246): diagonal columns, identical
// columns, and gap runs (maximal runs of same-orientation gap moves).
//
// The walk follows the DP's own decisions, so its path is the one whose
// statistics dp_warp carries to the end cell: H-state cells move as their
// source says (diagonal, or into the F / E gap state of the same cell), a gap
// state moves one row up (F) or one column left (E) and returns to H-state
// when its gap was opened.  Borders: a global alignment reaching row 0 or
// column 0 finishes along it in one gap run; a local alignment stops there,
// or at a cell whose H fell to 0, and starts at that cell.
#pragma once
#include <cstdint>

#include "../../include/pastis_gb300.h"
#include "pg_dpdir.cuh"

namespace pg {

struct TraceOut {
    uint32_t M, D, G;
    int i0, j0;
};

// The direction words of a region as a walk reads them: word (s * (n + VL -
// 1) + k) * VL + v of stripe s, step k, lane v (VL = 32 lanes, or 64 virtual
// lanes).  A walk only moves to smaller k and smaller v, so a miss loads a
// tile of TK steps x 4 lanes ending at the missed word (TK independent 16-byte
// loads, one memory round trip) and the next steps read it from the tile
// until the walk leaves it: about TK steps per round trip instead of one.
template <int VL>
struct DirTile {
    static constexpr int TK = 8;
    const uint32_t *dir;
    int n;
    uint4 t[TK];
    int ts = -1, tk0 = 0, tvb = -1;
    __device__ __forceinline__ DirTile(const uint32_t *d, int n_) : dir(d), n(n_) {}
    __device__ __forceinline__ uint32_t get(int s, int k, int v)
    {
        const int vb = v & ~3;
        if (s != ts || vb != tvb || k > tk0 || k <= tk0 - TK) {
            ts = s; tvb = vb; tk0 = k;
            const uint4 *b = reinterpret_cast<const uint4 *>(dir + (uint64_t)s * (uint64_t)(n + VL - 1) * VL + vb);
#pragma unroll
            for (int q = 0; q < TK; ++q)
                t[q] = k - q >= 0 ? __ldg(b + (uint64_t)(k - q) * (VL / 4)) : make_uint4(0u, 0u, 0u, 0u);
        }
        const uint4 w = t[tk0 - k];
        const int c = v - vb;
        return c == 0 ? w.x : (c == 1 ? w.y : (c == 2 ? w.z : w.w));
    }
};

template <bool LOCAL>
__device__ TraceOut trace_back(const uint32_t *__restrict__ dir, int n, int R, int i, int j,
                               const uint8_t *__restrict__ V, const uint8_t *__restrict__ Hs)
{
    uint32_t M = 0, D = 0, G = 0;
    int state = 0;   // 0: H, 1: F (vertical gap), 2: E (horizontal gap)
    int last = 0;    // orientation of the previous move: 0 diagonal / none, 1 vertical, 2 horizontal
    const int rows = 32 * R;
    DirTile<32> tile(dir, n);
    for (;;) {
        if (i == 0 || j == 0) {
            if (!LOCAL) {
                if (i > 0 && last != 1) ++G;
                else if (j > 0 && last != 2) ++G;
            }
            break;
        }
        const int r0 = i - 1;
        const int stripe = r0 / rows, within = r0 - stripe * rows;
        const int lane = within / R, r = within - lane * R;
        const uint32_t w = tile.get(stripe, j - 1 + lane, lane);
        const uint32_t nib = (w >> (4 * r)) & 15u;
        if (state == 0) {
            const uint32_t hs = nib & 3u;
            if (hs == DIR_ZERO) break;
            if (hs == DIR_DIAG) {
                ++D;
                M += __ldg(V + i - 1) == __ldg(Hs + j - 1) ? 1u : 0u;
                --i; --j;
                last = 0;
                continue;
            }
            state = hs == DIR_F ? 1 : 2;
        }
        if (state == 1) {
            if (last != 1) ++G;
            last = 1;
            state = (nib & DIR_FOPEN) ? 0 : 1;
            --i;
        } else {
            if (last != 2) ++G;
            last = 2;
            state = (nib & DIR_EOPEN) ? 0 : 2;
            --j;
        }
    }
    TraceOut o;
    o.M = M; o.D = D; o.G = G; o.i0 = i; o.j0 = j;
    return o;
}

// Traceback over the nibbles of dp_warp_dir16 (pg_dpdir16.cuh): the same walk
// and counts as trace_back.  Bit 0 of a nibble says H is not the diagonal,
// bit 1 then picks E over F; a local walk carries the value of the state it
// stands on (h: the end cell's score, less each diagonal's substitution score,
// plus the gap score a gap move undoes) and stops at an H-state cell whose
// value is 0, the cells the 32-bit form marks with its zero code.  sm is the
// PG_NRES x PG_NRES substitution table.
template <bool LOCAL>
__device__ TraceOut trace_back16(const uint32_t *__restrict__ dir, int n, int R, int i, int j,
                                 const uint8_t *__restrict__ V, const uint8_t *__restrict__ Hs,
                                 const int8_t *__restrict__ sm, int go, int ge, int h)
{
    uint32_t M = 0, D = 0, G = 0;
    int state = 0;   // 0: H, 1: F (vertical gap), 2: E (horizontal gap)
    int last = 0;    // orientation of the previous move: 0 diagonal / none, 1 vertical, 2 horizontal
    const int rows = 64 * R;
    DirTile<64> tile(dir, n);
    for (;;) {
        if (i == 0 || j == 0) {
            if (!LOCAL) {
                if (i > 0 && last != 1) ++G;
                else if (j > 0 && last != 2) ++G;
            }
            break;
        }
        if (LOCAL && state == 0 && h == 0) break;
        const int r0 = i - 1;
        const int stripe = r0 / rows, within = r0 - stripe * rows;
        const int v = within / R, r = within - v * R;
        const uint32_t w = tile.get(stripe, j - 1 + v, v);
        const uint32_t nib = (w >> (4 * r)) & 15u;
        if (state == 0) {
            if (!(nib & 1u)) {
                const int a = __ldg(V + i - 1), b = __ldg(Hs + j - 1);
                ++D;
                M += a == b ? 1u : 0u;
                if (LOCAL) h -= (a < PG_NRES && b < PG_NRES) ? (int)__ldg(sm + a * PG_NRES + b) : 0;
                --i; --j;
                last = 0;
                continue;
            }
            state = (nib & 2u) ? 2 : 1;
        }
        if (state == 1) {
            if (last != 1) ++G;
            last = 1;
            const bool open = (nib & DIR_FOPEN) != 0;
            if (LOCAL) h -= open ? go : ge;
            state = open ? 0 : 1;
            --i;
        } else {
            if (last != 2) ++G;
            last = 2;
            const bool open = (nib & DIR_EOPEN) != 0;
            if (LOCAL) h -= open ? go : ge;
            state = open ? 0 : 2;
            --j;
        }
    }
    TraceOut o;
    o.M = M; o.D = D; o.G = G; o.i0 = i; o.j0 = j;
    return o;
}

}  // namespace pg
