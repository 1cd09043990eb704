// pg_kmer.cu -- candidate generation on the GPU: the k-mer SpGEMM C = A·Aᵀ of
// PASTIS (src/kmer/KmerOps.cpp:31-245, src/sim_search.cpp:154-187) with the
// KmerIntersectLoc semiring (inc/sr.hpp:30-117), restated as sort and join.
//
//   1. k-mers of every row and column sequence of the block: code over the
//      alphabet (Horner, base = alphabet size, as KmerOps.cpp:60-62), offset;
//      one warp per sequence, lanes across positions.
//   2. radix sort of each side by code (the columns of A).
//   3. join: every row occurrence meets the run of equal codes on the column
//      side; each occurrence pair that survives the symmetric prune becomes a
//      product (key = col << 32 | row, seed = code << 32 | row off << 16 | col off).
//   4. radix sort of the products by key, run-length encoding, and per pair:
//      count = run length, first / second seed = smallest / largest seed
//      value, score = largest k-mer self score; ckthr / mosthr applied.
// The products of one call live in HBM at once (16 B each plus the sort's
// double buffer); max_products bounds them and callers block larger inputs,
// as PASTIS blocks its SpGEMM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include "../../include/pastis_gb300.h"

int pg_internal_seqs(const pg_ctx *c, const uint8_t **rseq, const uint64_t **roffs, uint64_t *nr,
                     const uint8_t **cseq, const uint64_t **coffs, uint64_t *nc, int *device,
                     void **stream, int *mode);
int pg_internal_fail(int code, const char *msg);
int pg_internal_score(const pg_ctx *c, const int8_t **d_sm);

namespace {

#define KCU(call)                                                                  \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return pg_internal_fail(e_ == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, \
                                    cudaGetErrorString(e_));                       \
    } while (0)

// murphy10 code of each residue code (ARNDCQEGHILKMFPSTWYVBZX*J): codes in the
// order Alphabet::init assigns them (src/Alphabet.cpp:31-51) to the groups of
// inc/Alphabet.hpp:83-104; the representative residue of each murphy10 code.
constexpr uint8_t kMurphy[PG_NRES] = {0, 1, 2, 2, 3, 2, 2, 4, 5, 6, 6, 1, 6, 7, 8, 9, 9, 7, 7, 6,
                                      10, 11, 12, 13, 14};
constexpr uint8_t kMurphyRep[15] = {0, 11, 3, 4, 7, 8, 9, 13, 14, 15, 20, 21, 22, 23, 24};

struct KmerTab {
    uint8_t map[32];     // residue code -> alphabet code
    int16_t cost[32];    // alphabet code -> self score of its letter
    uint32_t base;
    int k;
};

// k-mers of sequences [s0, s0 + ns) of one side; one warp per sequence
__global__ void k_kmer_fill(const uint8_t *seq, const uint64_t *offs, uint64_t s0, uint64_t ns,
                            int stride, const uint64_t *start, KmerTab tab, uint32_t *codes,
                            uint64_t *vals)
{
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint64_t s = warp; s < ns; s += nwarps) {
        const uint64_t b = offs[s0 + s];
        const int len = (int)(offs[s0 + s + 1] - b);
        if (len < tab.k) continue;
        const int nk = (len - tab.k) / stride + 1;
        const uint64_t o = start[s];
        for (int q = lane; q < nk; q += 32) {
            const int pos = q * stride;
            uint32_t code = 0;
            for (int j = 0; j < tab.k; ++j) code = code * tab.base + tab.map[seq[b + pos + j] & 31];
            codes[o + q] = code;
            vals[o + q] = (s << 16) | (uint64_t)pos;
        }
    }
}

__global__ void k_kmer_count(const uint64_t *offs, uint64_t s0, uint64_t ns, int k, int stride,
                             uint64_t *cnt)
{
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const int len = (int)(offs[s0 + s + 1] - offs[s0 + s]);
        cnt[s] = len < k ? 0 : (uint64_t)((len - k) / stride + 1);
    }
}

// first index in [lo, hi) with a[i] >= v
__device__ __forceinline__ uint64_t lower(const uint32_t *a, uint64_t lo, uint64_t hi, uint32_t v)
{
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// PG_PRUNE_* on global indices (sim_search.cpp:172-186 and :403-412)
__device__ __forceinline__ bool keep_pair(int prune, uint64_t r, uint64_t c)
{
    if (prune == PG_PRUNE_EVEN_ODD) {
        if (r == c) return false;
        const bool odd = ((r ^ c) & 1) != 0;
        return r > c ? !odd : odd;
    }
    if (prune == PG_PRUNE_UPPER) return r < c;
    return true;
}

// pass 1 (emit == false): products per row occurrence; pass 2: write them
template <bool EMIT>
__global__ void k_join(const uint32_t *rcode, const uint64_t *rval, uint64_t nrk,
                       const uint32_t *ccode, const uint64_t *cval, uint64_t nck,
                       uint64_t row_begin, uint64_t col_begin, int prune, uint64_t *cnt,
                       const uint64_t *start, uint64_t *keys, uint64_t *seeds)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrk;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t code = rcode[i];
        const uint64_t lo = lower(ccode, 0, nck, code);
        const uint64_t rv = rval[i];
        const uint64_t r = rv >> 16, rpos = rv & 0xffff;
        uint64_t n = 0, o = EMIT ? start[i] : 0;
        for (uint64_t j = lo; j < nck && ccode[j] == code; ++j) {
            const uint64_t cv = cval[j];
            const uint64_t c = cv >> 16, cpos = cv & 0xffff;
            if (!keep_pair(prune, r + row_begin, c + col_begin)) continue;
            if (EMIT) {
                keys[o] = (c << 32) | r;
                seeds[o] = ((uint64_t)code << 32) | (rpos << 16) | cpos;
                ++o;
            } else {
                ++n;
            }
        }
        if (!EMIT) cnt[i] = n;
    }
}

// one pair per run of equal keys
__global__ void k_reduce_pairs(const uint64_t *ukeys, const uint32_t *rlen, const uint64_t *rstart,
                               const uint64_t *nruns, const uint64_t *seeds, KmerTab tab,
                               int ckthr, int mosthr, pg_pair *out, uint32_t *keep)
{
    const uint64_t nr = *nruns;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nr;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = rstart[u];
        const uint32_t len = rlen[u];
        uint64_t mn = ~0ull, mx = 0;
        int score = -32768;
        for (uint32_t q = 0; q < len; ++q) {
            const uint64_t sv = seeds[b + q];
            mn = sv < mn ? sv : mn;
            mx = sv > mx ? sv : mx;
            uint32_t code = (uint32_t)(sv >> 32);
            int cost = 0;
            for (int j = 0; j < tab.k; ++j) { cost += tab.cost[code % tab.base]; code /= tab.base; }
            score = cost > score ? cost : score;
        }
        const uint16_t count = (uint16_t)len;   // ushort arithmetic of the semiring
        pg_pair p;
        p.row = (uint32_t)(ukeys[u] & 0xffffffffu);
        p.col = (uint32_t)(ukeys[u] >> 32);
        p.rs0 = (uint16_t)((mn >> 16) & 0xffff);
        p.cs0 = (uint16_t)(mn & 0xffff);
        p.rs1 = len >= 2 ? (uint16_t)((mx >> 16) & 0xffff) : 0;
        p.cs1 = len >= 2 ? (uint16_t)(mx & 0xffff) : 0;
        p.count = count;
        p.score = (int16_t)score;
        out[u] = p;
        keep[u] = ((int)count > ckthr && score > mosthr) ? 1u : 0u;
    }
}

__global__ void k_triple_flags(const pg_result *res, uint64_t n, uint32_t *keep)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (uint64_t)gridDim.x * blockDim.x)
        keep[i] = (i < n && res[i].score_aln != 0.0f) ? 1u : 0u;
}

__global__ void k_triple_write(const pg_pair *pairs, const pg_result *res, uint64_t n,
                               const uint32_t *keep, const uint64_t *pos, uint64_t roff,
                               uint64_t coff, uint64_t *rows, uint64_t *cols, float *vals)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        const uint64_t o = pos[i];
        rows[o] = (uint64_t)pairs[i].row + roff;
        cols[o] = (uint64_t)pairs[i].col + coff;
        vals[o] = res[i].score_aln;
    }
}

__global__ void k_compact_pairs(const pg_pair *in, const uint32_t *keep, const uint64_t *pos,
                                const uint64_t *nruns, pg_pair *out)
{
    const uint64_t nr = *nruns;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nr;
         u += (uint64_t)gridDim.x * blockDim.x)
        if (keep[u]) out[pos[u]] = in[u];
}

// device buffers of one call, freed on every exit path
struct Bufs {
    std::vector<void *> ptrs;
    cudaStream_t st = nullptr;
    ~Bufs()
    {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    template <class T>
    cudaError_t get(T **p, size_t count)
    {
        void *q = nullptr;
        const cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(count * sizeof(T), 16), st);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
};

uint64_t pow_u(uint64_t b, int k)
{
    uint64_t r = 1;
    for (int i = 0; i < k; ++i) r *= b;
    return r;
}

struct SideKmers {
    uint32_t *code = nullptr;
    uint64_t *val = nullptr;
    uint64_t n = 0;
};

int side_kmers(Bufs &B, const uint8_t *seq, const uint64_t *offs, uint64_t s0, uint64_t ns,
               const pg_kmer_config &kc, const KmerTab &tab, int nsm, SideKmers &out)
{
    cudaStream_t st = B.st;
    uint64_t *cnt, *start;
    KCU(B.get(&cnt, ns + 1));
    KCU(B.get(&start, ns + 1));
    const int grid = nsm * 8;
    KCU(cudaMemsetAsync(cnt + ns, 0, sizeof(uint64_t), st));
    k_kmer_count<<<grid, 256, 0, st>>>(offs, s0, ns, kc.k, kc.stride, cnt);
    size_t tb = 0;
    KCU(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, start, ns + 1, st));
    void *tmp;
    KCU(B.get((char **)&tmp, tb));
    KCU(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, start, ns + 1, st));
    uint64_t total = 0;
    KCU(cudaMemcpyAsync(&total, start + ns, sizeof total, cudaMemcpyDeviceToHost, st));
    KCU(cudaStreamSynchronize(st));
    out.n = total;
    uint32_t *c0, *c1;
    uint64_t *v0, *v1;
    KCU(B.get(&c0, total)); KCU(B.get(&c1, total));
    KCU(B.get(&v0, total)); KCU(B.get(&v1, total));
    if (total) k_kmer_fill<<<grid, 256, 0, st>>>(seq, offs, s0, ns, kc.stride, start, tab, c0, v0);
    KCU(cudaGetLastError());
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < pow_u(tab.base, tab.k)) ++bits;
    cub::DoubleBuffer<uint32_t> kb(c0, c1);
    cub::DoubleBuffer<uint64_t> vb(v0, v1);
    size_t sb = 0;
    KCU(cub::DeviceRadixSort::SortPairs(nullptr, sb, kb, vb, (int64_t)total, 0, bits, st));
    void *stmp;
    KCU(B.get((char **)&stmp, sb));
    KCU(cub::DeviceRadixSort::SortPairs(stmp, sb, kb, vb, (int64_t)total, 0, bits, st));
    out.code = kb.Current();
    out.val = vb.Current();
    return PG_OK;
}

}  // namespace

extern "C" {

void pg_kmer_config_default(pg_kmer_config *kc)
{
    if (!kc) return;
    std::memset(kc, 0, sizeof *kc);
    kc->k = 6;
    kc->stride = 1;
    kc->alphabet = PG_ALPH_PROTEIN;
    kc->prune = PG_PRUNE_NONE;
    kc->ckthr = 0;          // src/main.cpp:104-105
    kc->mosthr = -1;
    kc->max_products = 0;
}

int pg_candidates(pg_ctx *ctx, const pg_kmer_config *kc, uint64_t row_begin, uint64_t row_end,
                  uint64_t col_begin, uint64_t col_end, pg_pair *d_out, uint64_t cap,
                  uint64_t *n_out, void *stream)
{
    if (!ctx || !kc || !n_out || (cap && !d_out))
        return pg_internal_fail(PG_ERR_ARG, "pg_candidates: bad argument");
    *n_out = 0;
    if (kc->k < 1 || kc->k > 16 || kc->stride < 1 || (kc->alphabet != PG_ALPH_PROTEIN &&
        kc->alphabet != PG_ALPH_MURPHY10) || kc->prune < 0 || kc->prune > 2)
        return pg_internal_fail(PG_ERR_ARG, "pg_candidates: bad k-mer configuration");
    const uint8_t *rseq, *cseq;
    const uint64_t *roffs, *coffs;
    uint64_t nr, nc;
    int dev, mode;
    void *cst;
    int rc = pg_internal_seqs(ctx, &rseq, &roffs, &nr, &cseq, &coffs, &nc, &dev, &cst, &mode);
    if (rc) return rc;
    if (row_begin > row_end || row_end > nr || col_begin > col_end || col_end > nc)
        return pg_internal_fail(PG_ERR_ARG, "pg_candidates: block out of range");
    if (row_end - row_begin >= (1ull << 32) || col_end - col_begin >= (1ull << 32))
        return pg_internal_fail(PG_ERR_ARG, "pg_candidates: block wider than 2^32 sequences");
    const int8_t *d_sm = nullptr;
    rc = pg_internal_score(ctx, &d_sm);
    if (rc) return rc;
    KmerTab tab;
    std::memset(&tab, 0, sizeof tab);
    tab.k = kc->k;
    int8_t sm[PG_NRES * PG_NRES];
    KCU(cudaSetDevice(dev));
    KCU(cudaMemcpy(sm, d_sm, sizeof sm, cudaMemcpyDeviceToHost));
    if (kc->alphabet == PG_ALPH_PROTEIN) {
        tab.base = PG_NRES;
        for (int a = 0; a < PG_NRES; ++a) { tab.map[a] = (uint8_t)a; tab.cost[a] = sm[a * PG_NRES + a]; }
    } else {
        tab.base = 15;
        for (int a = 0; a < PG_NRES; ++a) tab.map[a] = kMurphy[a];
        for (int m = 0; m < 15; ++m) tab.cost[m] = sm[kMurphyRep[m] * PG_NRES + kMurphyRep[m]];
    }
    for (int a = PG_NRES; a < 32; ++a) tab.map[a] = tab.map[22];   // out-of-table codes read as X
    // the reference asserts the k-mer universe fits an int (KmerOps.cpp:117-120)
    if (pow_u(tab.base, tab.k) > (uint64_t)0x7fffffff)
        return pg_internal_fail(PG_ERR_ARG, "pg_candidates: alphabet^k exceeds 2^31");
    int nsm = 0;
    KCU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    Bufs B;
    B.st = stream ? (cudaStream_t)stream : (cudaStream_t)cst;
    cudaStream_t st = B.st;
    SideKmers R, C;
    rc = side_kmers(B, rseq, roffs, row_begin, row_end - row_begin, *kc, tab, nsm, R);
    if (rc) return rc;
    const bool same = rseq == cseq && roffs == coffs && row_begin == col_begin && row_end == col_end;
    if (same) C = R;
    else {
        rc = side_kmers(B, cseq, coffs, col_begin, col_end - col_begin, *kc, tab, nsm, C);
        if (rc) return rc;
    }
    const int grid = nsm * 8;
    // products per row occurrence, then their offsets
    uint64_t *pcnt, *pstart;
    KCU(B.get(&pcnt, R.n + 1));
    KCU(B.get(&pstart, R.n + 1));
    KCU(cudaMemsetAsync(pcnt + R.n, 0, sizeof(uint64_t), st));
    if (R.n)
        k_join<false><<<grid, 256, 0, st>>>(R.code, R.val, R.n, C.code, C.val, C.n, row_begin,
                                            col_begin, kc->prune, pcnt, nullptr, nullptr, nullptr);
    KCU(cudaGetLastError());
    size_t tb = 0;
    KCU(cub::DeviceScan::ExclusiveSum(nullptr, tb, pcnt, pstart, R.n + 1, st));
    void *tmp;
    KCU(B.get((char **)&tmp, tb));
    KCU(cub::DeviceScan::ExclusiveSum(tmp, tb, pcnt, pstart, R.n + 1, st));
    uint64_t P = 0;
    KCU(cudaMemcpyAsync(&P, pstart + R.n, sizeof P, cudaMemcpyDeviceToHost, st));
    KCU(cudaStreamSynchronize(st));
    const uint64_t maxp = kc->max_products ? kc->max_products : (1ull << 31);
    if (P > maxp) return pg_internal_fail(PG_ERR_RANGE, "pg_candidates: too many k-mer occurrence pairs for one block");
    if (P == 0) return PG_OK;
    uint64_t *k0, *k1, *s0, *s1;
    KCU(B.get(&k0, P)); KCU(B.get(&k1, P));
    KCU(B.get(&s0, P)); KCU(B.get(&s1, P));
    k_join<true><<<grid, 256, 0, st>>>(R.code, R.val, R.n, C.code, C.val, C.n, row_begin, col_begin,
                                       kc->prune, nullptr, pstart, k0, s0);
    KCU(cudaGetLastError());
    int cbits = 1;
    while (cbits < 32 && (1ull << cbits) < (col_end - col_begin)) ++cbits;
    cub::DoubleBuffer<uint64_t> kb(k0, k1), sb(s0, s1);
    size_t sbytes = 0;
    KCU(cub::DeviceRadixSort::SortPairs(nullptr, sbytes, kb, sb, (int64_t)P, 0, 32 + cbits, st));
    void *stmp;
    KCU(B.get((char **)&stmp, sbytes));
    KCU(cub::DeviceRadixSort::SortPairs(stmp, sbytes, kb, sb, (int64_t)P, 0, 32 + cbits, st));
    // runs of equal keys = candidate pairs
    uint64_t *ukeys, *nruns, *rstart;
    uint32_t *rlen, *keep;
    KCU(B.get(&ukeys, P)); KCU(B.get(&rlen, P + 1)); KCU(B.get(&nruns, 1));
    KCU(B.get(&rstart, P + 1)); KCU(B.get(&keep, P + 1));
    size_t eb = 0;
    KCU(cub::DeviceRunLengthEncode::Encode(nullptr, eb, kb.Current(), ukeys, rlen, nruns, (int64_t)P, st));
    void *etmp;
    KCU(B.get((char **)&etmp, eb));
    KCU(cub::DeviceRunLengthEncode::Encode(etmp, eb, kb.Current(), ukeys, rlen, nruns, (int64_t)P, st));
    uint64_t U = 0;
    KCU(cudaMemcpyAsync(&U, nruns, sizeof U, cudaMemcpyDeviceToHost, st));
    KCU(cudaStreamSynchronize(st));
    KCU(cudaMemsetAsync(rlen + U, 0, sizeof(uint32_t), st));
    size_t xb = 0;
    KCU(cub::DeviceScan::ExclusiveSum(nullptr, xb, rlen, rstart, (int64_t)(U + 1), st));
    void *xtmp;
    KCU(B.get((char **)&xtmp, xb));
    KCU(cub::DeviceScan::ExclusiveSum(xtmp, xb, rlen, rstart, (int64_t)(U + 1), st));
    pg_pair *all;
    KCU(B.get(&all, U));
    k_reduce_pairs<<<grid, 256, 0, st>>>(ukeys, rlen, rstart, nruns, sb.Current(), tab, kc->ckthr,
                                         kc->mosthr, all, keep);
    KCU(cudaGetLastError());
    uint64_t *kpos;
    KCU(B.get(&kpos, U + 1));
    KCU(cudaMemsetAsync(keep + U, 0, sizeof(uint32_t), st));
    size_t qb = 0;
    KCU(cub::DeviceScan::ExclusiveSum(nullptr, qb, keep, kpos, (int64_t)(U + 1), st));
    void *qtmp;
    KCU(B.get((char **)&qtmp, qb));
    KCU(cub::DeviceScan::ExclusiveSum(qtmp, qb, keep, kpos, (int64_t)(U + 1), st));
    uint64_t K = 0;
    KCU(cudaMemcpyAsync(&K, kpos + U, sizeof K, cudaMemcpyDeviceToHost, st));
    KCU(cudaStreamSynchronize(st));
    *n_out = K;
    if (K > cap) return pg_internal_fail(PG_ERR_RANGE, "pg_candidates: output capacity too small");
    k_compact_pairs<<<grid, 256, 0, st>>>(all, keep, kpos, nruns, d_out);
    KCU(cudaGetLastError());
    KCU(cudaStreamSynchronize(st));
    return PG_OK;
}

int pg_triples(const pg_pair *d_pairs, const pg_result *d_res, uint64_t n, uint64_t bl_roffset,
               uint64_t bl_coffset, uint64_t *d_rows, uint64_t *d_cols, float *d_vals,
               uint64_t *n_out, void *stream)
{
    if (!n_out || (n && (!d_pairs || !d_res || !d_rows || !d_cols || !d_vals)))
        return pg_internal_fail(PG_ERR_ARG, "pg_triples: bad argument");
    *n_out = 0;
    if (!n) return PG_OK;
    int dev = 0, nsm = 0;
    KCU(cudaGetDevice(&dev));
    KCU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    Bufs B;
    B.st = (cudaStream_t)stream;
    uint32_t *keep;
    uint64_t *pos;
    KCU(B.get(&keep, n + 1));
    KCU(B.get(&pos, n + 1));
    const int grid = nsm * 8;
    k_triple_flags<<<grid, 256, 0, B.st>>>(d_res, n, keep);
    size_t tb = 0;
    KCU(cub::DeviceScan::ExclusiveSum(nullptr, tb, keep, pos, n + 1, B.st));
    void *tmp;
    KCU(B.get((char **)&tmp, tb));
    KCU(cub::DeviceScan::ExclusiveSum(tmp, tb, keep, pos, n + 1, B.st));
    k_triple_write<<<grid, 256, 0, B.st>>>(d_pairs, d_res, n, keep, pos, bl_roffset, bl_coffset,
                                            d_rows, d_cols, d_vals);
    KCU(cudaGetLastError());
    uint64_t cnt = 0;
    KCU(cudaMemcpyAsync(&cnt, pos + n, sizeof cnt, cudaMemcpyDeviceToHost, B.st));
    KCU(cudaStreamSynchronize(B.st));
    *n_out = cnt;
    return PG_OK;
}

}  // extern "C"
