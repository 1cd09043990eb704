// pg_fasta.cu -- FASTA ingest on the GPU straight into a context's resident,
// encoded sequences, replacing the host parse of FastaData::FastaData
// (src/FastaData.cpp:13-148) and the copy into seqan::Peptide strings
// (src/align/SeqanFullAligner.cpp:28-88).
//
// The reference's character state machine, restated in parallel:
//   - a record starts at the first '>' of a line (a later '>' on the same
//     line is inside the name);
//   - its sequence text runs from the line after the header to the next
//     record; newlines and '*' are dropped, 'U' / 'u' become 'T';
//   - a record with fewer than k residues is removed where the reference
//     checks: when the next record starts right after a newline of the
//     sequence text, and for the last record.
//   1. newline positions (flag + scan + scatter);
//   2. one thread per line finds its first '>';
//   3. one warp per record counts residues, applies the removal rule;
//   4. one warp per kept record encodes its residues into place.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include "../../include/pastis_gb300.h"

int pg_internal_fail(int code, const char *msg);
int pg_internal_adopt_side(pg_ctx *c, int side, uint8_t *d_codes, uint64_t *d_offs, uint64_t n,
                           uint32_t maxlen);
int pg_internal_device(const pg_ctx *c, int *device, void **stream);

namespace {

#define FCU_(call)                                                                 \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return pg_internal_fail(e_ == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, \
                                    cudaGetErrorString(e_));                       \
    } while (0)

constexpr unsigned FULLM = 0xffffffffu;

struct Enc {
    uint8_t t[256];
};

Enc make_enc()
{
    Enc e;
    const char *letters = "ARNDCQEGHILKMFPSTWYVBZX*J";
    for (int i = 0; i < 256; ++i) e.t[i] = 22;   // X
    for (int i = 0; i < PG_NRES; ++i) {
        e.t[(unsigned char)letters[i]] = (uint8_t)i;
        if (letters[i] >= 'A' && letters[i] <= 'Z') e.t[(unsigned char)(letters[i] - 'A' + 'a')] = (uint8_t)i;
    }
    return e;
}

__global__ void k_nl_flags(const char *buf, uint64_t L, uint32_t *flag)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= L;
         i += (uint64_t)gridDim.x * blockDim.x)
        flag[i] = (i < L && buf[i] == '\n') ? 1u : 0u;
}

__global__ void k_nl_scatter(const uint32_t *flag, const uint64_t *pos, uint64_t L, uint64_t *nl)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (flag[i]) nl[pos[i]] = i;
}

// line j = [start, end): start = 0 or nl[j-1] + 1, end = nl[j] or L.
// hdr[j] = position of its first '>' or ~0
__global__ void k_line_hdr(const char *buf, uint64_t L, const uint64_t *nl, uint64_t nlines,
                           uint64_t *hdr, uint32_t *has)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j <= nlines;
         j += (uint64_t)gridDim.x * blockDim.x) {
        if (j == nlines) { has[j] = 0; continue; }
        const uint64_t s = j ? nl[j - 1] + 1 : 0;
        const uint64_t e = j + 1 < nlines ? nl[j] : L;
        uint64_t h = ~0ull;
        for (uint64_t q = s; q < e; ++q)
            if (buf[q] == '>') { h = q; break; }
        hdr[j] = h;
        has[j] = h != ~0ull ? 1u : 0u;
    }
}

__global__ void k_hdr_scatter(const uint64_t *hdr, const uint32_t *has, const uint64_t *pos,
                              uint64_t nlines, const uint64_t *nl, uint64_t L, uint64_t *H,
                              uint64_t *name_end)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nlines;
         j += (uint64_t)gridDim.x * blockDim.x)
        if (has[j]) {
            H[pos[j]] = hdr[j];
            name_end[pos[j]] = j + 1 < nlines ? nl[j] : L;   // L: the name is the last line
        }
}

// residues and removal per record; one warp per record
__global__ void k_rec_count(const char *buf, uint64_t L, const uint64_t *H, const uint64_t *name_end,
                            uint64_t nrec, int k, uint64_t *len, uint32_t *keep)
{
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint64_t r = warp; r <= nrec; r += nwarps) {
        if (r == nrec) { if (lane == 0) { len[r] = 0; keep[r] = 0; } continue; }
        const uint64_t ne = name_end[r];
        const uint64_t next = r + 1 < nrec ? H[r + 1] : L;
        const uint64_t s = ne < L ? ne + 1 : L;
        uint64_t cnt = 0;
        for (uint64_t q0 = s; q0 < next; q0 += 32) {
            const uint64_t q = q0 + lane;
            const bool res = q < next && buf[q] != '\n' && buf[q] != '*';
            cnt += __popc(__ballot_sync(FULLM, res));
        }
        if (lane == 0) {
            bool checked = r + 1 == nrec;
            if (!checked) {
                const uint64_t b = next - 1;   // the character before the next record
                checked = buf[b] == '\n' && b != ne;
            }
            len[r] = cnt;
            keep[r] = (checked && cnt < (uint64_t)k) ? 0u : 1u;
        }
    }
}

// kept record u (original r = kidx[u]) into codes[off[u] ...)
__global__ void k_rec_fill(const char *buf, uint64_t L, const uint64_t *H, const uint64_t *name_end,
                           uint64_t nrec, const uint64_t *kidx, uint64_t nk, const uint64_t *off,
                           Enc enc, uint8_t *codes)
{
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint64_t u = warp; u < nk; u += nwarps) {
        const uint64_t r = kidx[u];
        const uint64_t ne = name_end[r];
        const uint64_t next = r + 1 < nrec ? H[r + 1] : L;
        const uint64_t s = ne < L ? ne + 1 : L;
        uint64_t o = off[u];
        for (uint64_t q0 = s; q0 < next; q0 += 32) {
            const uint64_t q = q0 + lane;
            const char ch = q < next ? buf[q] : '\n';
            const bool res = ch != '\n' && ch != '*';
            const unsigned m = __ballot_sync(FULLM, res);
            if (res) {
                const char t = (ch == 'U' || ch == 'u') ? 'T' : ch;
                codes[o + __popc(m & ((1u << lane) - 1u))] = enc.t[(unsigned char)t];
            }
            o += __popc(m);
        }
    }
}

__global__ void k_kept_index(const uint32_t *keep, const uint64_t *kpos, uint64_t nrec,
                             const uint64_t *len, uint64_t *kidx, uint64_t *klen)
{
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrec;
         r += (uint64_t)gridDim.x * blockDim.x)
        if (keep[r]) { kidx[kpos[r]] = r; klen[kpos[r]] = len[r]; }
}

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

template <class In, class Out>
int excl_sum(Bufs &B, const In *in, Out *out, uint64_t n)
{
    size_t tb = 0;
    FCU_(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, n, B.st));
    void *tmp;
    FCU_(B.get((char **)&tmp, tb));
    FCU_(cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, n, B.st));
    return PG_OK;
}

}  // namespace

extern "C" int pg_set_seqs_fasta(pg_ctx *ctx, int32_t side, const char *fasta, uint64_t len,
                                 int32_t k, uint64_t *n_kept, uint64_t *n_removed,
                                 uint64_t *orig_index, uint64_t orig_cap)
{
    if (!ctx || (side != 0 && side != 1) || (len && !fasta) || k < 0)
        return pg_internal_fail(PG_ERR_ARG, "pg_set_seqs_fasta: bad argument");
    int dev = 0;
    void *cst = nullptr;
    int rc = pg_internal_device(ctx, &dev, &cst);
    if (rc) return rc;
    FCU_(cudaSetDevice(dev));
    uint64_t L = len;
    while (L && fasta[L - 1] == '\n') --L;   // the reference's l_end: last real character
    int nsm = 0;
    FCU_(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int grid = nsm * 8;
    Bufs B;
    B.st = (cudaStream_t)cst;
    cudaStream_t st = B.st;
    char *d_buf;
    FCU_(B.get(&d_buf, L + 1));
    if (L) FCU_(cudaMemcpyAsync(d_buf, fasta, L, cudaMemcpyHostToDevice, st));
    // 1. newlines
    uint32_t *flag;
    uint64_t *fpos;
    FCU_(B.get(&flag, L + 1));
    FCU_(B.get(&fpos, L + 1));
    k_nl_flags<<<grid, 256, 0, st>>>(d_buf, L, flag);
    rc = excl_sum(B, flag, fpos, L + 1);
    if (rc) return rc;
    uint64_t nnl = 0;
    FCU_(cudaMemcpyAsync(&nnl, fpos + L, sizeof nnl, cudaMemcpyDeviceToHost, st));
    FCU_(cudaStreamSynchronize(st));
    uint64_t *nl;
    FCU_(B.get(&nl, nnl + 1));
    k_nl_scatter<<<grid, 256, 0, st>>>(flag, fpos, L, nl);
    const uint64_t nlines = L ? nnl + 1 : 0;
    // 2. record starts
    uint64_t *hdr, *hpos;
    uint32_t *has;
    FCU_(B.get(&hdr, nlines + 1));
    FCU_(B.get(&has, nlines + 1));
    FCU_(B.get(&hpos, nlines + 1));
    k_line_hdr<<<grid, 256, 0, st>>>(d_buf, L, nl, nlines, hdr, has);
    rc = excl_sum(B, has, hpos, nlines + 1);
    if (rc) return rc;
    uint64_t nrec = 0;
    FCU_(cudaMemcpyAsync(&nrec, hpos + nlines, sizeof nrec, cudaMemcpyDeviceToHost, st));
    FCU_(cudaStreamSynchronize(st));
    uint64_t *H, *name_end;
    FCU_(B.get(&H, nrec + 1));
    FCU_(B.get(&name_end, nrec + 1));
    k_hdr_scatter<<<grid, 256, 0, st>>>(hdr, has, hpos, nlines, nl, L, H, name_end);
    // 3. residues per record and the removal rule
    uint64_t *rlen, *kpos;
    uint32_t *keep;
    FCU_(B.get(&rlen, nrec + 1));
    FCU_(B.get(&keep, nrec + 1));
    FCU_(B.get(&kpos, nrec + 1));
    k_rec_count<<<grid, 256, 0, st>>>(d_buf, L, H, name_end, nrec, k, rlen, keep);
    rc = excl_sum(B, keep, kpos, nrec + 1);
    if (rc) return rc;
    uint64_t nk = 0;
    FCU_(cudaMemcpyAsync(&nk, kpos + nrec, sizeof nk, cudaMemcpyDeviceToHost, st));
    FCU_(cudaStreamSynchronize(st));
    uint64_t *kidx, *klen;
    FCU_(B.get(&kidx, nk + 1));
    FCU_(B.get(&klen, nk + 1));
    FCU_(cudaMemsetAsync(klen + nk, 0, sizeof(uint64_t), st));
    k_kept_index<<<grid, 256, 0, st>>>(keep, kpos, nrec, rlen, kidx, klen);
    // 4. offsets, longest sequence, residues
    uint64_t *d_offs = nullptr;
    FCU_(cudaMalloc(&d_offs, (nk + 1) * sizeof(uint64_t)));
    rc = excl_sum(B, klen, d_offs, nk + 1);
    if (rc) { cudaFree(d_offs); return rc; }
    uint64_t *d_max;
    FCU_(B.get(&d_max, 1));
    size_t mb = 0;
    FCU_(cub::DeviceReduce::Max(nullptr, mb, klen, d_max, nk + 1, st));
    void *mtmp;
    FCU_(B.get((char **)&mtmp, mb));
    FCU_(cub::DeviceReduce::Max(mtmp, mb, klen, d_max, nk + 1, st));
    uint64_t total = 0, maxlen = 0;
    FCU_(cudaMemcpyAsync(&total, d_offs + nk, sizeof total, cudaMemcpyDeviceToHost, st));
    FCU_(cudaMemcpyAsync(&maxlen, d_max, sizeof maxlen, cudaMemcpyDeviceToHost, st));
    FCU_(cudaStreamSynchronize(st));
    if (maxlen > 65535) {
        cudaFree(d_offs);
        return pg_internal_fail(PG_ERR_RANGE, "pg_set_seqs_fasta: a sequence has more than 65535 residues");
    }
    uint8_t *d_codes = nullptr;
    if (cudaMalloc(&d_codes, total ? total : 1) != cudaSuccess) {
        cudaFree(d_offs);
        return pg_internal_fail(PG_ERR_OOM, "pg_set_seqs_fasta: residues");
    }
    if (nk) k_rec_fill<<<grid, 256, 0, st>>>(d_buf, L, H, name_end, nrec, kidx, nk, d_offs, make_enc(), d_codes);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && orig_index && nk)
        e = cudaMemcpyAsync(orig_index, kidx, std::min(nk, orig_cap) * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(d_offs); cudaFree(d_codes);
        return pg_internal_fail(PG_ERR_CUDA, cudaGetErrorString(e));
    }
    if (n_kept) *n_kept = nk;
    if (n_removed) *n_removed = nrec - nk;
    return pg_internal_adopt_side(ctx, side, d_codes, d_offs, nk, (uint32_t)maxlen);
}
