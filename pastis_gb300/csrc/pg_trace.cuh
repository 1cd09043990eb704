// pg_trace.cuh -- traceback over the direction nibbles of dp_warp_dir
// (pg_dpdir.cuh, 32 lanes) or dp_warp_dir16 / dp_pair_dir16 (pg_dpdir16.cuh,
// 64 or 32 virtual lanes): a walk from the region's end cell back to its start that counts
// what computeAlignmentStats counts (src/align/SeqanFullAligner.cpp:238-246):
// diagonal columns, identical columns, and gap runs (maximal runs of
// same-orientation gap moves).
//
// The walk follows the DP's own decisions, so its path is the one whose
// statistics dp_warp carries to the end cell: H-state cells move as their
// source says (diagonal, or into the F / E gap state of the same cell), a gap
// state moves one row up (F) or one column left (E) and returns to H-state
// when its gap was opened.  Borders: a global alignment reaching row 0 or
// column 0 finishes along it in one gap run; a local alignment stops there,
// or at a cell whose H fell to 0, and starts at that cell.
//
// One thread walks one region, one 4-byte direction word per step (the
// words sit in HBM: the DP of a whole chunk writes them first).  Two
// read-ahead schemes measured slower and were dropped: a per-thread tile of
// 8 steps x 4 lanes (a refill somewhere in the warp at nearly every step,
// and 8 sectors read per refill), and one warp per region reading 32-step x
// 8-lane tiles through shuffles (a 32nd of the walks in flight).
#pragma once
#include <cstdint>

#include "../../include/pastis_gb300.h"
#include "pg_dpdir.cuh"
#include "pg_dpdir16.cuh"

namespace pg {

struct TraceOut {
    uint32_t M, D, G;
    int i0, j0;
};

// A walker over one region.  W16: the nibbles of dp_warp_dir16 or
// dp_pair_dir16 (bit 0: not the diagonal, bit 1: E rather than F; a local walk
// carries the score of the cell it stands on, h, and stops where it is 0).
// Otherwise the nibbles of dp_warp_dir (bits 0-1: diagonal, F, E or the local
// floor).  Words: (s * (n + vl - 1) + k) * vl + v for stripe s, wavefront step
// k = j - 1 + v, lane v (vl = 32 lanes of dp_warp_dir); the 16-bit regions
// lie in 4-step tiles (dir16_pair_word for the half-warp regions of
// dp_pair_dir16, vl = 32; dir16_warp_word for the whole-warp ones, vl = 64).  ssm: the 32 x 32 substitution table in shared memory (read only
// by a local W16 walk).  step() makes one move and returns false once the walk
// has ended; the counts are then final.
template <bool LOCAL, bool W16>
struct Walker {
    const uint32_t *dir;
    const uint8_t *V, *Hs;
    const int *ssm;
    int n, R, vl, go, ge;
    int i, j, h;
    int s = 0, v = 0, r = 0;   // row i - 1 as stripe, lane, row of the lane (kept in step with i)
    int state = 0;             // 0: H, 1: F (vertical gap), 2: E (horizontal gap)
    int last = 0;              // previous move: 0 diagonal / none, 1 vertical, 2 horizontal
    uint32_t M = 0, D = 0, G = 0;
    bool done = false;

    __device__ __forceinline__ Walker(const uint32_t *dir_, int n_, int R_, int vl_, int i_, int j_,
                                      const uint8_t *V_, const uint8_t *Hs_, const int *ssm_,
                                      int go_, int ge_, int h_)
        : dir(dir_), V(V_), Hs(Hs_), ssm(ssm_), n(n_), R(R_), vl(vl_), go(go_), ge(ge_), i(i_), j(j_),
          h(h_)
    {
        if (i > 0) {
            const int r0 = i - 1, rows = vl * R;
            s = r0 / rows;
            const int within = r0 - s * rows;
            v = within / R;
            r = within - v * R;
        }
    }
    __device__ __forceinline__ void up()
    {
        if (--r < 0) {
            r = R - 1;
            if (--v < 0) { v = vl - 1; --s; }
        }
    }
    __device__ __forceinline__ bool step()
    {
        if (done) return false;
        if (i == 0 || j == 0) {
            if (!LOCAL) {
                if (i > 0 && last != 1) ++G;
                else if (j > 0 && last != 2) ++G;
            }
            done = true;
            return false;
        }
        // the word of (i, j) first (i, j >= 1 here): its load does not wait on h,
        // whose substitution-score lookups it overlaps
        const uint64_t widx = !W16 ? ((uint64_t)s * (uint64_t)(n + vl - 1) + (uint64_t)(j - 1 + v)) * (uint64_t)vl + v
                              : vl == 32 ? dir16_pair_word(j - 1 + v, v) : dir16_warp_word(s, j - 1 + v, v, n);
        const uint32_t w = __ldg(dir + widx);
        {
            // the walk moves back through the wavefront steps: ask L1 now for
            // the word 1 KiB back in either layout (8 steps of the half-warp
            // tiles, 4 steps of the others), so that its sector is there when
            // the walk arrives (sw100k 9.13 -> 9.02 ms per step; xdrop1m
            // alignment 40.27 -> 40.16 ms with every 16-bit region tiled)
            const uint64_t back = (W16 && vl == 32) ? 256u : 4u * (uint64_t)vl;
            if (widx >= back) asm volatile("prefetch.global.L1 [%0];" :: "l"(dir + widx - back));
        }
        if (W16 && LOCAL && state == 0 && h == 0) { done = true; return false; }
        const uint32_t nib = (w >> (4 * r)) & 15u;
        if (state == 0) {
            bool diag;
            if (W16) {
                diag = !(nib & 1u);
                if (!diag) state = (nib & 2u) ? 2 : 1;
            } else {
                const uint32_t hs = nib & 3u;
                if (hs == DIR_ZERO) { done = true; return false; }
                diag = hs == DIR_DIAG;
                if (!diag) state = hs == DIR_F ? 1 : 2;
            }
            if (diag) {
                const int a = __ldg(V + i - 1), b = __ldg(Hs + j - 1);
                ++D;
                M += a == b ? 1u : 0u;
                if (W16 && LOCAL) h -= ssm[a * 32 + b];
                --i; --j;
                up();
                last = 0;
                return true;
            }
        }
        const bool open = (nib & (state == 1 ? DIR_FOPEN : DIR_EOPEN)) != 0;
        if (W16 && LOCAL) h -= open ? go : ge;
        if (state == 1) {
            if (last != 1) ++G;
            last = 1;
            --i;
            up();
        } else {
            if (last != 2) ++G;
            last = 2;
            --j;
        }
        if (open) state = 0;
        return true;
    }
    __device__ __forceinline__ TraceOut out() const
    {
        TraceOut o;
        o.M = M; o.D = D; o.G = G; o.i0 = i; o.j0 = j;
        return o;
    }
};

template <bool LOCAL, bool W16>
__device__ __forceinline__ TraceOut trace_walk(const uint32_t *dir, int n, int R, int vl, int i, int j,
                                               const uint8_t *V, const uint8_t *Hs, const int *ssm,
                                               int go, int ge, int h)
{
    Walker<LOCAL, W16> w(dir, n, R, vl, i, j, V, Hs, ssm, go, ge, h);
    while (w.step()) {}
    return w.out();
}

}  // namespace pg
