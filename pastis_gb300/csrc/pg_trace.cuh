// pg_trace.cuh -- traceback over the direction nibbles of dp_warp_dir
// (pg_dpdir.cuh, 32 lanes) or dp_warp_dir16 (pg_dpdir16.cuh, 64 virtual
// lanes): a walk from the region's end cell back to its start that counts
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
// One warp walks one region, every lane the same walk (uniform control
// flow).  A walk is a chain of dependent reads, one per step, so the warp
// reads ahead in tiles: the direction words of 32 wavefront steps x 8 lanes
// (one 16-byte load per lane, one memory round trip) and 128 residues of
// each sequence (4 per lane); each step takes its word or residue from the
// tile with a shuffle, and only a step that leaves a tile pays a round trip
// (a walk moves to smaller steps, lanes and residues only).  One thread per
// region with a word load per step measured slower: every step waited on
// memory, and a per-thread tile misses somewhere in the warp at nearly every
// step.
#pragma once
#include <cstdint>

#include "../../include/pastis_gb300.h"
#include "pg_dpdir.cuh"

namespace pg {

struct TraceOut {
    uint32_t M, D, G;
    int i0, j0;
};

// Direction words of a region: word (s * (n + VL - 1) + k) * VL + v of stripe
// s, wavefront step k, lane v (VL = 32 lanes, or 64 virtual lanes).  Lane L
// holds the 4 words of lanes vb + 4 (L & 1) .. + 3 at steps k0 - (L >> 1) and
// k0 - 16 - (L >> 1).
template <int VL>
struct WarpDirTile {
    const uint32_t *dir;
    int n;
    uint4 a, b;
    int ts = -1, tk0 = 0, tvb = -1;
    __device__ __forceinline__ WarpDirTile(const uint32_t *d, int n_) : dir(d), n(n_) {}
    __device__ __forceinline__ uint32_t get(int s, int k, int v)
    {
        const int vb = v & ~7;
        if (s != ts || vb != tvb || k > tk0 || k < tk0 - 31) {
            ts = s; tvb = vb; tk0 = k;
            const int lane = threadIdx.x & 31;
            const uint32_t *row = dir + (uint64_t)s * (uint64_t)(n + VL - 1) * VL + vb + 4 * (lane & 1);
            const int k1 = k - (lane >> 1), k2 = k1 - 16;
            a = k1 >= 0 ? __ldg(reinterpret_cast<const uint4 *>(row + (uint64_t)k1 * VL)) : make_uint4(0u, 0u, 0u, 0u);
            b = k2 >= 0 ? __ldg(reinterpret_cast<const uint4 *>(row + (uint64_t)k2 * VL)) : make_uint4(0u, 0u, 0u, 0u);
        }
        const int d = v - vb, idx = tk0 - k;
        const uint4 q = idx < 16 ? a : b;
        const int c = d & 3;
        const uint32_t mine = c == 0 ? q.x : (c == 1 ? q.y : (c == 2 ? q.z : q.w));
        return __shfl_sync(FULL, mine, ((idx & 15) << 1) | (d >> 2));
    }
};

// residues [base, base + 128) of a sequence of len residues, 4 per lane
struct WarpResidues {
    const uint8_t *seq;
    int len;
    uint32_t w = 0;
    int base = -(1 << 30);
    __device__ __forceinline__ WarpResidues(const uint8_t *s, int l) : seq(s), len(l) {}
    __device__ __forceinline__ int get(int p)     // 0 <= p < len
    {
        if (p < base || p >= base + 128) {
            base = p >= 127 ? p - 127 : 0;        // walks move to smaller p
            const int q0 = base + 4 * (threadIdx.x & 31);
            uint32_t x = 0;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (q0 + c < len) x |= (uint32_t)__ldg(seq + q0 + c) << (8 * c);
            w = x;
        }
        const int d = p - base;
        return (int)((__shfl_sync(FULL, w, d >> 2) >> (8 * (d & 3))) & 0xffu);
    }
};

// The walk, called by all 32 lanes with the same arguments; every lane
// returns the same counts.  W16: the nibbles of dp_warp_dir16 (bit 0: not the
// diagonal, bit 1: E rather than F; a local walk carries the score of the
// cell it stands on, h, and stops where it is 0).  Otherwise the nibbles of
// dp_warp_dir (bits 0-1: diagonal, F, E or the local floor).  ssm: the 32 x
// 32 substitution table in shared memory (read only by a local W16 walk).
template <bool LOCAL, bool W16>
__device__ TraceOut trace_walk(const uint32_t *__restrict__ dir, int n, int R, int i, int j,
                               const uint8_t *__restrict__ V, int m, const uint8_t *__restrict__ Hs,
                               const int *__restrict__ ssm, int go, int ge, int h)
{
    constexpr int VL = W16 ? 64 : 32;
    uint32_t M = 0, D = 0, G = 0;
    int state = 0;   // 0: H, 1: F (vertical gap), 2: E (horizontal gap)
    int last = 0;    // orientation of the previous move: 0 diagonal / none, 1 vertical, 2 horizontal
    WarpDirTile<VL> tile(dir, n);
    WarpResidues rv(V, m), rh(Hs, n);
    // row i - 1 as stripe s, lane v, row r of the lane (kept in step with i)
    int s = 0, v = 0, r = 0;
    if (i > 0) {
        const int r0 = i - 1, rows = VL * R;
        s = r0 / rows;
        const int within = r0 - s * rows;
        v = within / R;
        r = within - v * R;
    }
    auto up = [&]() {
        if (--r < 0) {
            r = R - 1;
            if (--v < 0) { v = VL - 1; --s; }
        }
    };
    for (;;) {
        if (i == 0 || j == 0) {
            if (!LOCAL) {
                if (i > 0 && last != 1) ++G;
                else if (j > 0 && last != 2) ++G;
            }
            break;
        }
        if (W16 && LOCAL && state == 0 && h == 0) break;
        const uint32_t nib = (tile.get(s, j - 1 + v, v) >> (4 * r)) & 15u;
        if (state == 0) {
            bool diag;
            if (W16) {
                diag = !(nib & 1u);
                if (!diag) state = (nib & 2u) ? 2 : 1;
            } else {
                const uint32_t hs = nib & 3u;
                if (hs == DIR_ZERO) break;
                diag = hs == DIR_DIAG;
                if (!diag) state = hs == DIR_F ? 1 : 2;
            }
            if (diag) {
                const int a = rv.get(i - 1), b = rh.get(j - 1);
                ++D;
                M += a == b ? 1u : 0u;
                if (W16 && LOCAL) h -= ssm[a * 32 + b];
                --i; --j;
                up();
                last = 0;
                continue;
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
    }
    TraceOut o;
    o.M = M; o.D = D; o.G = G; o.i0 = i; o.j0 = j;
    return o;
}

}  // namespace pg
