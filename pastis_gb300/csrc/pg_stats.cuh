// pg_stats.cuh -- packed path statistics carried through the DP.
//
// A statistics value travels with the predecessor a traceback would choose
// (see pg_dp.cuh) and holds what computeAlignmentStats reports for the traced
// alignment: matches M, diagonal columns D, gap runs G and, for local
// alignment, the first aligned residue (i0, j0).  Packing is chosen per region
// size so the common case costs one register and one select per choice:
//
//   S1   M | D << 10 | G << 20            regions up to 1023 x 1023 (G <= m + n)
//   S2   M | D << 16, G                   regions up to 65535 x 65535
//   L1   M | D << 10 | G << 20, i0 | j0 << 16     local, both sides <= 1023
//   L2   M | D << 16, G, i0 | j0 << 16            local, any size
#pragma once
#include <cstdint>

namespace pg {

struct S1 {
    uint32_t w;
    static constexpr bool LOCAL = false;
    static constexpr int MAXSIDE = 1023;
    __device__ __forceinline__ static S1 zero() { return S1{0}; }
    __device__ __forceinline__ static S1 gap1() { return S1{1u << 20}; }
    __device__ __forceinline__ static S1 sel(bool p, const S1 &a, const S1 &b) { return S1{p ? a.w : b.w}; }
    __device__ __forceinline__ S1 diag(uint32_t match) const { return S1{w + (1u << 10) + match}; }
    __device__ __forceinline__ S1 open() const { return S1{w + (1u << 20)}; }
    __device__ __forceinline__ static S1 reset(int, int) { return S1{0}; }
    __device__ __forceinline__ S1 shfl_up() const { return S1{__shfl_up_sync(0xffffffffu, w, 1)}; }
    __device__ __forceinline__ S1 shfl(int src) const { return S1{__shfl_sync(0xffffffffu, w, src)}; }
    __device__ __forceinline__ S1 shfl_xor(int o) const { return S1{__shfl_xor_sync(0xffffffffu, w, o)}; }
    __device__ __forceinline__ uint32_t M() const { return w & 1023u; }
    __device__ __forceinline__ uint32_t D() const { return (w >> 10) & 1023u; }
    __device__ __forceinline__ uint32_t G() const { return w >> 20; }
    __device__ __forceinline__ int i0() const { return 0; }
    __device__ __forceinline__ int j0() const { return 0; }
};

struct S2 {
    uint32_t md, g;
    static constexpr bool LOCAL = false;
    static constexpr int MAXSIDE = 65535;
    __device__ __forceinline__ static S2 zero() { return S2{0, 0}; }
    __device__ __forceinline__ static S2 gap1() { return S2{0, 1}; }
    __device__ __forceinline__ static S2 sel(bool p, const S2 &a, const S2 &b)
    {
        return S2{p ? a.md : b.md, p ? a.g : b.g};
    }
    __device__ __forceinline__ S2 diag(uint32_t match) const { return S2{md + (1u << 16) + match, g}; }
    __device__ __forceinline__ S2 open() const { return S2{md, g + 1}; }
    __device__ __forceinline__ static S2 reset(int, int) { return S2{0, 0}; }
    __device__ __forceinline__ S2 shfl_up() const
    {
        return S2{__shfl_up_sync(0xffffffffu, md, 1), __shfl_up_sync(0xffffffffu, g, 1)};
    }
    __device__ __forceinline__ S2 shfl(int src) const
    {
        return S2{__shfl_sync(0xffffffffu, md, src), __shfl_sync(0xffffffffu, g, src)};
    }
    __device__ __forceinline__ S2 shfl_xor(int o) const
    {
        return S2{__shfl_xor_sync(0xffffffffu, md, o), __shfl_xor_sync(0xffffffffu, g, o)};
    }
    __device__ __forceinline__ uint32_t M() const { return md & 0xffffu; }
    __device__ __forceinline__ uint32_t D() const { return md >> 16; }
    __device__ __forceinline__ uint32_t G() const { return g; }
    __device__ __forceinline__ int i0() const { return 0; }
    __device__ __forceinline__ int j0() const { return 0; }
};

struct L1 {
    uint32_t w, b;
    static constexpr bool LOCAL = true;
    static constexpr int MAXSIDE = 1023;
    __device__ __forceinline__ static L1 zero() { return L1{0, 0}; }
    __device__ __forceinline__ static L1 gap1() { return L1{1u << 20, 0}; }
    __device__ __forceinline__ static L1 sel(bool p, const L1 &a, const L1 &c)
    {
        return L1{p ? a.w : c.w, p ? a.b : c.b};
    }
    __device__ __forceinline__ L1 diag(uint32_t match) const { return L1{w + (1u << 10) + match, b}; }
    __device__ __forceinline__ L1 open() const { return L1{w + (1u << 20), b}; }
    __device__ __forceinline__ static L1 reset(int i, int j) { return L1{0, (uint32_t)i | ((uint32_t)j << 16)}; }
    __device__ __forceinline__ L1 shfl_up() const
    {
        return L1{__shfl_up_sync(0xffffffffu, w, 1), __shfl_up_sync(0xffffffffu, b, 1)};
    }
    __device__ __forceinline__ L1 shfl(int src) const
    {
        return L1{__shfl_sync(0xffffffffu, w, src), __shfl_sync(0xffffffffu, b, src)};
    }
    __device__ __forceinline__ L1 shfl_xor(int o) const
    {
        return L1{__shfl_xor_sync(0xffffffffu, w, o), __shfl_xor_sync(0xffffffffu, b, o)};
    }
    __device__ __forceinline__ uint32_t M() const { return w & 1023u; }
    __device__ __forceinline__ uint32_t D() const { return (w >> 10) & 1023u; }
    __device__ __forceinline__ uint32_t G() const { return w >> 20; }
    __device__ __forceinline__ int i0() const { return (int)(b & 0xffffu); }
    __device__ __forceinline__ int j0() const { return (int)(b >> 16); }
};

struct L2 {
    uint32_t md, g, b;
    static constexpr bool LOCAL = true;
    static constexpr int MAXSIDE = 65535;
    __device__ __forceinline__ static L2 zero() { return L2{0, 0, 0}; }
    __device__ __forceinline__ static L2 gap1() { return L2{0, 1, 0}; }
    __device__ __forceinline__ static L2 sel(bool p, const L2 &a, const L2 &c)
    {
        return L2{p ? a.md : c.md, p ? a.g : c.g, p ? a.b : c.b};
    }
    __device__ __forceinline__ L2 diag(uint32_t match) const { return L2{md + (1u << 16) + match, g, b}; }
    __device__ __forceinline__ L2 open() const { return L2{md, g + 1, b}; }
    __device__ __forceinline__ static L2 reset(int i, int j) { return L2{0, 0, (uint32_t)i | ((uint32_t)j << 16)}; }
    __device__ __forceinline__ L2 shfl_up() const
    {
        return L2{__shfl_up_sync(0xffffffffu, md, 1), __shfl_up_sync(0xffffffffu, g, 1),
                  __shfl_up_sync(0xffffffffu, b, 1)};
    }
    __device__ __forceinline__ L2 shfl(int src) const
    {
        return L2{__shfl_sync(0xffffffffu, md, src), __shfl_sync(0xffffffffu, g, src),
                  __shfl_sync(0xffffffffu, b, src)};
    }
    __device__ __forceinline__ L2 shfl_xor(int o) const
    {
        return L2{__shfl_xor_sync(0xffffffffu, md, o), __shfl_xor_sync(0xffffffffu, g, o),
                  __shfl_xor_sync(0xffffffffu, b, o)};
    }
    __device__ __forceinline__ uint32_t M() const { return md & 0xffffu; }
    __device__ __forceinline__ uint32_t D() const { return md >> 16; }
    __device__ __forceinline__ uint32_t G() const { return g; }
    __device__ __forceinline__ int i0() const { return (int)(b & 0xffffu); }
    __device__ __forceinline__ int j0() const { return (int)(b >> 16); }
};

}  // namespace pg
