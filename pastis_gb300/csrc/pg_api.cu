// pg_api.cu -- C ABI of the GB300 batched pairwise aligner (declared in
// include/pastis_gb300.h).  Host side: sequence residency, scratch sizing,
// launch of the persistent kernels in pg_kernels.cuh, error reporting.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/pastis_gb300.h"
#include <cub/device/device_scan.cuh>

#include "pg_dir.h"
#include "pg_stat.h"
#include "pg_kernels.cuh"
#include "pg_kernels_xd.cuh"

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

#define CU(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                 \
    } while (0)

// Published BLOSUM62 in PASTIS's residue order ARNDCQEGHILKMFPSTWYVBZX*J
// (src/Alphabet.cpp:26); J scores as L, as in inc/ScoreMat.hpp:104-131.
const signed char kB62[24][24] = {
    { 4,-1,-2,-2, 0,-1,-1, 0,-2,-1,-1,-1,-1,-2,-1, 1, 0,-3,-2, 0,-2,-1, 0,-4},
    {-1, 5, 0,-2,-3, 1, 0,-2, 0,-3,-2, 2,-1,-3,-2,-1,-1,-3,-2,-3,-1, 0,-1,-4},
    {-2, 0, 6, 1,-3, 0, 0, 0, 1,-3,-3, 0,-2,-3,-2, 1, 0,-4,-2,-3, 3, 0,-1,-4},
    {-2,-2, 1, 6,-3, 0, 2,-1,-1,-3,-4,-1,-3,-3,-1, 0,-1,-4,-3,-3, 4, 1,-1,-4},
    { 0,-3,-3,-3, 9,-3,-4,-3,-3,-1,-1,-3,-1,-2,-3,-1,-1,-2,-2,-1,-3,-3,-2,-4},
    {-1, 1, 0, 0,-3, 5, 2,-2, 0,-3,-2, 1, 0,-3,-1, 0,-1,-2,-1,-2, 0, 3,-1,-4},
    {-1, 0, 0, 2,-4, 2, 5,-2, 0,-3,-3, 1,-2,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1,-4},
    { 0,-2, 0,-1,-3,-2,-2, 6,-2,-4,-4,-2,-3,-3,-2, 0,-2,-2,-3,-3,-1,-2,-1,-4},
    {-2, 0, 1,-1,-3, 0, 0,-2, 8,-3,-3,-1,-2,-1,-2,-1,-2,-2, 2,-3, 0, 0,-1,-4},
    {-1,-3,-3,-3,-1,-3,-3,-4,-3, 4, 2,-3, 1, 0,-3,-2,-1,-3,-1, 3,-3,-3,-1,-4},
    {-1,-2,-3,-4,-1,-2,-3,-4,-3, 2, 4,-2, 2, 0,-3,-2,-1,-2,-1, 1,-4,-3,-1,-4},
    {-1, 2, 0,-1,-3, 1, 1,-2,-1,-3,-2, 5,-1,-3,-1, 0,-1,-3,-2,-2, 0, 1,-1,-4},
    {-1,-1,-2,-3,-1, 0,-2,-3,-2, 1, 2,-1, 5, 0,-2,-1,-1,-1,-1, 1,-3,-1,-1,-4},
    {-2,-3,-3,-3,-2,-3,-3,-3,-1, 0, 0,-3, 0, 6,-4,-2,-2, 1, 3,-1,-3,-3,-1,-4},
    {-1,-2,-2,-1,-3,-1,-1,-2,-2,-3,-3,-1,-2,-4, 7,-1,-1,-4,-3,-2,-2,-1,-2,-4},
    { 1,-1, 1, 0,-1, 0, 0, 0,-1,-2,-2, 0,-1,-2,-1, 4, 1,-3,-2,-2, 0, 0, 0,-4},
    { 0,-1, 0,-1,-1,-1,-1,-2,-2,-1,-1,-1,-1,-2,-1, 1, 5,-2,-2, 0,-1,-1, 0,-4},
    {-3,-3,-4,-4,-2,-2,-3,-2,-2,-3,-2,-3,-1, 1,-4,-3,-2,11, 2,-3,-4,-3,-2,-4},
    {-2,-2,-2,-3,-2,-1,-2,-3, 2,-1,-1,-2,-1, 3,-3,-2,-2, 2, 7,-1,-3,-2,-1,-4},
    { 0,-3,-3,-3,-1,-2,-2,-3,-3, 3, 1,-2, 1,-1,-2,-2, 0,-3,-1, 4,-3,-2,-1,-4},
    {-2,-1, 3, 4,-3, 0, 1,-1, 0,-3,-4, 0,-3,-3,-2, 0,-1,-4,-3,-3, 4, 1,-1,-4},
    {-1, 0, 0, 1,-3, 3, 4,-2, 0,-3,-3, 1,-1,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1,-4},
    { 0,-1,-1,-1,-2,-1,-1,-1,-1,-1,-1,-1,-1,-1,-2, 0, 0,-2,-1,-1,-1,-1,-1,-4},
    {-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4, 1},
};

void blosum62(int8_t *out)
{
    for (int a = 0; a < PG_NRES; ++a)
        for (int b = 0; b < PG_NRES; ++b) {
            const int aa = a == 24 ? 10 : a, bb = b == 24 ? 10 : b;
            out[a * PG_NRES + b] = (int8_t)kB62[aa][bb];
        }
}

struct Encoder {
    uint8_t t[256];
    Encoder()
    {
        const char *letters = "ARNDCQEGHILKMFPSTWYVBZX*J";
        for (int i = 0; i < 256; ++i) t[i] = 22;  // X
        for (int i = 0; i < PG_NRES; ++i) {
            t[(unsigned char)letters[i]] = (uint8_t)i;
            if (letters[i] >= 'A' && letters[i] <= 'Z')
                t[(unsigned char)(letters[i] - 'A' + 'a')] = (uint8_t)i;
        }
    }
};
const Encoder kEnc;

struct Side {
    uint8_t *seq = nullptr;
    uint64_t *offs = nullptr;
    uint64_t n = 0;
    uint64_t nres = 0;      // residues of all its sequences
    uint32_t maxlen = 0;
};

size_t next_pow2(size_t x)
{
    size_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

}  // namespace

struct pg_ctx {
    pg_config cfg{};
    int go = 0, ge = 0, xg = 0;
    int8_t sm[PG_NRES * PG_NRES];
    int8_t *d_sm = nullptr;
    cudaStream_t stream = nullptr;
    int nsm = 0;
    int grid = 0;                  // persistent blocks of the warp-per-pair kernel
    int grid_xd = 0;               // persistent blocks of k_xdf
    int grid_xd_run = 0;           // persistent blocks of k_xd
    int grid_xdr = 0;              // persistent blocks of k_xdr
    uint64_t l2_bytes = 0;         // the device's L2 cache
    int grid_wide = 0;             // blocks of k_xd_wide
    Side side[2];
    bool cols_share_rows = false;
    // scratch
    unsigned int *d_counter = nullptr;  // 4 work counters, then the bucket schedule words
    int *d_status = nullptr;
    unsigned long long *d_exec = nullptr;
    void *d_bnd = nullptr;              // per-warp DP row scratch
    uint64_t bnd_bytes = 0;             // bytes per warp
    size_t bnd_warps = 0;
    int *d_gring = nullptr;             // per-warp X-drop fallback ring
    int gring_w = 0;
    size_t gring_warps = 0;
    pg::XdRec *d_xd = nullptr;          // 2 extension records per pair
    uint32_t *d_ovf = nullptr;          // overflowed extension tasks
    uint64_t xd_cap = 0;
    uint32_t *d_order = nullptr;        // bucket order of the pairs
    uint32_t *d_xorder = nullptr;       // X-drop extension tasks, longest length bound first
    uint64_t order_cap = 0;
    // traceback form: direction arena, per-task byte counts / offsets,
    // per-pair scores and end cells, scan scratch
    uint8_t *d_dir = nullptr;
    uint64_t dir_cap = 0, dir_budget = 0;
    uint64_t *d_dbytes = nullptr, *d_doff = nullptr, *d_t1 = nullptr;
    int *d_dsc = nullptr;
    void *d_scan = nullptr;
    size_t scan_bytes = 0;
    uint64_t dirb_cap = 0;
    // staging for the host-buffer entry point
    pg_pair *d_pairs = nullptr;
    pg_result *d_out = nullptr;
    uint64_t cap = 0;
    int last_launches = 0;
    // timing of the last batch: [0] start, [1] extension done, [2] alignment done
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    bool events_valid = false;
    // launch tuning and the captured graph of the last batch shape
    pg_tuning tune{};
    int dp_per_sm = 1, xd_per_sm = 1;   // occupancy limits
    int lim16 = 0;                      // largest m + n for 16-bit lanes (dp_traceback 2 and 3)
    uint64_t epoch = 0;                 // bumped whenever a buffer a graph holds moves
    cudaGraphExec_t gexec = nullptr;
    struct GraphKey {
        const void *pairs, *out;
        uint64_t n, roff, coff, epoch;
        cudaStream_t st;
        bool operator==(const GraphKey &o) const
        {
            return pairs == o.pairs && out == o.out && n == o.n && roff == o.roff &&
                   coff == o.coff && epoch == o.epoch && st == o.st;
        }
    } gkey{};
    int graph_launches = 0;
    bool capturing = false;             // launch() is being recorded into a graph
};

extern "C" {

void pg_config_default(pg_config *cfg, int32_t mode)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->mode = mode;
    cfg->gap_open = -11;
    cfg->gap_ext = -2;
    cfg->gap_semantics = PG_GAPS_AS_CALLED;
    cfg->xdrop = 49;
    cfg->seed_len = 6;
    cfg->seed_count = 2;
    cfg->tie = 0;
    cfg->flags = 0;
    cfg->ani_thr = 30;
    cfg->cov_thr = 0.7;
    cfg->device = 0;
    cfg->score_matrix = nullptr;
}

const char *pg_strerror(int code)
{
    switch (code) {
    case PG_OK: return "ok";
    case PG_ERR_ARG: return "invalid argument";
    case PG_ERR_CUDA: return "CUDA error";
    case PG_ERR_OOM: return "out of memory";
    case PG_ERR_STATE: return "invalid call order";
    case PG_ERR_RANGE: return "sequence longer than 65535 residues";
    case PG_ERR_NODEV: return "no usable CUDA device";
    default: return "unknown error";
    }
}

const char *pg_last_error(void) { return g_err; }

const char *pg_version(void) { return "pastis_gb300 0.1 (sm_103a)"; }

void pg_destroy(pg_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->cfg.device);
    for (int s = 0; s < 2; ++s) {
        if (s == 1 && ctx->cols_share_rows) break;
        cudaFree(ctx->side[s].seq);
        cudaFree(ctx->side[s].offs);
    }
    cudaFree(ctx->d_sm);
    cudaFree(ctx->d_counter);
    cudaFree(ctx->d_status);
    cudaFree(ctx->d_exec);
    cudaFree(ctx->d_bnd);
    cudaFree(ctx->d_gring);
    cudaFree(ctx->d_xd);
    cudaFree(ctx->d_ovf);
    cudaFree(ctx->d_order);
    cudaFree(ctx->d_xorder);
    cudaFree(ctx->d_dir); cudaFree(ctx->d_dbytes); cudaFree(ctx->d_doff); cudaFree(ctx->d_t1);
    cudaFree(ctx->d_dsc); cudaFree(ctx->d_scan);
    cudaFree(ctx->d_pairs);
    cudaFree(ctx->d_out);
    for (int k = 0; k < 3; ++k)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int validate(const pg_config *c)
{
    if (c->mode != PG_MODE_SW && c->mode != PG_MODE_XDROP) return fail(PG_ERR_ARG, "mode %d", c->mode);
    if (c->gap_semantics != PG_GAPS_AS_CALLED && c->gap_semantics != PG_GAPS_NOMINAL)
        return fail(PG_ERR_ARG, "gap_semantics %d", c->gap_semantics);
    if (c->gap_open < -1000 || c->gap_open > 1000 || c->gap_ext < -1000 || c->gap_ext > 1000)
        return fail(PG_ERR_ARG, "gap scores must lie in [-1000, 1000]");
    if (c->xdrop < 0 || c->xdrop > (1 << 28)) return fail(PG_ERR_ARG, "xdrop %d", c->xdrop);
    if (c->seed_len < 1 || c->seed_len > 65535) return fail(PG_ERR_ARG, "seed_len %d", c->seed_len);
    if (c->seed_count < 0) return fail(PG_ERR_ARG, "seed_count %d", c->seed_count);
    if (c->tie < 0 || c->tie > 3) return fail(PG_ERR_ARG, "tie %d", c->tie);
    if (c->flags & ~(PG_F_SKIP_SPURIOUS_SEED | PG_F_XDROP_AFFINE))
        return fail(PG_ERR_ARG, "flags %d", c->flags);
    return PG_OK;
}

int pg_create(const pg_config *cfg, pg_ctx **out)
{
    if (!cfg || !out) return fail(PG_ERR_ARG, "null argument");
    *out = nullptr;
    int rc = validate(cfg);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PG_ERR_NODEV, "no CUDA device");
    if (cfg->device < 0 || cfg->device >= ndev) return fail(PG_ERR_NODEV, "device %d of %d", cfg->device, ndev);
    CU(cudaSetDevice(cfg->device));
    pg_ctx *c = new (std::nothrow) pg_ctx();
    if (!c) return fail(PG_ERR_OOM, "host allocation");
    c->cfg = *cfg;
    c->cfg.score_matrix = nullptr;
    if (cfg->score_matrix) std::memcpy(c->sm, cfg->score_matrix, sizeof c->sm);
    else blosum62(c->sm);
    if (cfg->gap_semantics == PG_GAPS_AS_CALLED) {
        // seqan Score(gapExtend, gapOpen) receives (gap_open, gap_ext)
        c->go = cfg->gap_ext; c->ge = cfg->gap_open; c->xg = cfg->gap_open;
    } else {
        c->go = cfg->gap_open; c->ge = cfg->gap_ext; c->xg = cfg->gap_ext;
    }
    {
        // regions that the traceback form may run on 16-bit lanes
        int maxabs = std::max(std::abs(c->go), std::abs(c->ge));
        for (int k = 0; k < PG_NRES * PG_NRES; ++k) maxabs = std::max(maxabs, std::abs((int)c->sm[k]));
        c->lim16 = pg::dir16_limit(maxabs);
    }
#define CUD(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { pg_destroy(c); \
        return fail(e_ == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, "%s: %s", #call, \
                    cudaGetErrorString(e_)); } } while (0)
    CUD(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUD(cudaMalloc(&c->d_sm, sizeof c->sm));
    CUD(cudaMemcpy(c->d_sm, c->sm, sizeof c->sm, cudaMemcpyHostToDevice));
    CUD(cudaMalloc(&c->d_counter, (4 + pg::SCHED_WORDS + pg::XSCHED_WORDS) * sizeof(unsigned int)));
    CUD(cudaMalloc(&c->d_status, sizeof(int)));
    CUD(cudaMalloc(&c->d_exec, 2 * sizeof(unsigned long long)));
    CUD(cudaMemset(c->d_exec, 0, 2 * sizeof(unsigned long long)));
    for (int k = 0; k < 3; ++k) CUD(cudaEventCreate(&c->ev[k]));
    CUD(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, cfg->device));
    {
        int l2 = 0;
        CUD(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, cfg->device));
        c->l2_bytes = (uint64_t)l2;
    }
    CUD(pg::stat_set_attributes());
    CUD(pg::dir_set_attributes());
    {
        // the direction arena may take up to a third of the device memory
        size_t fr = 0, tot = 0;
        CUD(cudaMemGetInfo(&fr, &tot));
        c->dir_budget = std::max<uint64_t>((uint64_t)1 << 30, (uint64_t)tot / 3);
    }
    int per_sm = 0;
    if (cfg->mode == PG_MODE_XDROP) {
        CUD(pg::stat_occupancy(true, &per_sm));
        int px = 0, pw = 0;
        CUD(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&px, pg::k_xdf, pg::XT, 0));
        int pr = 0;
        CUD(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pr, pg::k_xd, pg::XT, 0));
        c->grid_xd_run = c->nsm * std::max(pr, 1);
        int pq = 0;
        CUD(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pq, pg::k_xdr<8>, pg::XT, 0));
        c->grid_xdr = c->nsm * std::max(pq, 1);
        CUD(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pw, pg::k_xd_wide, pg::WARPS * 32, 0));
        c->grid_xd = c->nsm * std::max(px, 1);
        c->grid_wide = c->nsm * std::max(pw, 1);
    } else {
        CUD(pg::stat_occupancy(false, &per_sm));
    }
    c->grid = c->nsm * std::max(per_sm, 1);
    c->dp_per_sm = std::max(per_sm, 1);
    c->xd_per_sm = c->grid_xd ? c->grid_xd / c->nsm : 1;
    pg_tuning_default(&c->tune);
    // The traceback form on 16-bit lanes measured fastest in both modes (DP
    // phase, sw100k: statistics 24.7 ms, 32-bit traceback 18.1 ms, 16-bit
    // 10.9 ms; xdrop1m: 72.8 / 78.6 / 57.9 ms).  With a score table too wide
    // for 16 bits every region would take 32-bit lanes, where the X-drop
    // global alignment is faster with statistics.
    c->tune.dp_traceback = c->lim16 > 0 ? 3 : (cfg->mode == PG_MODE_SW ? 1 : 0);
#undef CUD
    *out = c;
    return PG_OK;
}

// per-warp scratch for the current sequence set
static int ensure_scratch(pg_ctx *c)
{
    const uint32_t rmax = c->side[0].maxlen;
    const uint32_t cmax = c->cols_share_rows ? rmax : c->side[1].maxlen;
    // one DP row of the widest edge type (local statistics, 3 words)
    const size_t per_warp = ((size_t)cmax + 1) * sizeof(pg::Edge<pg::L2>);
    // keep the row scratch within 8 GiB: fewer resident warps for very long sequences
    size_t warps = (size_t)c->grid * pg::WARPS;
    const size_t budget = (size_t)8 << 30;
    if (per_warp * warps > budget) {
        warps = std::max<size_t>(pg::WARPS, budget / per_warp / pg::WARPS * pg::WARPS);
        c->grid = (int)(warps / pg::WARPS);
    }
    if (per_warp > c->bnd_bytes || warps > c->bnd_warps || !c->d_bnd) {
        cudaFree(c->d_bnd);
        c->d_bnd = nullptr;
        c->bnd_bytes = 0;
        ++c->epoch;
        CU(cudaMalloc(&c->d_bnd, per_warp * warps));
        c->bnd_bytes = per_warp;
        c->bnd_warps = warps;
    }
    if (c->cfg.mode == PG_MODE_XDROP) {
        const int gw = (int)next_pow2((size_t)std::max(rmax, cmax) + 4);
        const size_t wwarps = (size_t)c->grid_wide * pg::WARPS;
        // k_xd_wide keeps 3 anti-diagonals per warp, k_xda (affine gaps) 7
        const size_t arrays = (c->cfg.flags & PG_F_XDROP_AFFINE) ? pg::XDA_ARRAYS : 3;
        if (gw > c->gring_w || wwarps > c->gring_warps || !c->d_gring) {
            cudaFree(c->d_gring);
            c->d_gring = nullptr;
            c->gring_w = 0;
            ++c->epoch;
            CU(cudaMalloc(&c->d_gring, arrays * gw * sizeof(int) * wwarps));
            c->gring_w = gw;
            c->gring_warps = wwarps;
        }
    }
    return PG_OK;
}

// per-pair X-drop scratch for a batch of n pairs
static int ensure_batch(pg_ctx *c, uint64_t n)
{
    if (n > c->order_cap) {
        cudaFree(c->d_order);
        c->d_order = nullptr; c->order_cap = 0;
        ++c->epoch;
        CU(cudaMalloc(&c->d_order, n * sizeof(uint32_t)));
        c->order_cap = n;
    }
    if (c->cfg.mode != PG_MODE_XDROP || n <= c->xd_cap) return PG_OK;
    cudaFree(c->d_xd); cudaFree(c->d_ovf); cudaFree(c->d_xorder);
    c->d_xd = nullptr; c->d_ovf = nullptr; c->d_xorder = nullptr; c->xd_cap = 0;
    ++c->epoch;
    CU(cudaMalloc(&c->d_xd, 2 * n * sizeof(pg::XdRec)));
    CU(cudaMalloc(&c->d_ovf, 2 * n * sizeof(uint32_t)));
    CU(cudaMalloc(&c->d_xorder, 2 * n * sizeof(uint32_t)));
    c->xd_cap = n;
    return PG_OK;
}

int pg_set_seqs(pg_ctx *c, int32_t side, const char *residues, const uint64_t *offsets, uint64_t n)
{
    if (!c || (side != 0 && side != 1) || !offsets || (n > 0 && !residues))
        return fail(PG_ERR_ARG, "pg_set_seqs: bad argument");
    CU(cudaSetDevice(c->cfg.device));
    const uint64_t total = offsets[n] - offsets[0];
    uint32_t maxlen = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (offsets[i + 1] < offsets[i]) return fail(PG_ERR_ARG, "offsets not ascending at %llu", (unsigned long long)i);
        const uint64_t len = offsets[i + 1] - offsets[i];
        if (len > 65535) return fail(PG_ERR_RANGE, "sequence %llu has %llu residues", (unsigned long long)i, (unsigned long long)len);
        maxlen = std::max<uint32_t>(maxlen, (uint32_t)len);
    }
    uint8_t *codes = (uint8_t *)std::malloc(total ? total : 1);
    uint64_t *offs = (uint64_t *)std::malloc((n + 1) * sizeof(uint64_t));
    if (!codes || !offs) { std::free(codes); std::free(offs); return fail(PG_ERR_OOM, "host staging"); }
    const uint8_t *src = (const uint8_t *)residues + offsets[0];
    for (uint64_t q = 0; q < total; ++q) codes[q] = kEnc.t[src[q]];
    for (uint64_t i = 0; i <= n; ++i) offs[i] = offsets[i] - offsets[0];
    Side &s = c->side[side];
    if (side == 1 && c->cols_share_rows) { s = Side(); c->cols_share_rows = false; }
    if (side == 0 && c->cols_share_rows) { c->side[1] = Side(); c->cols_share_rows = false; }
    cudaFree(s.seq); cudaFree(s.offs);
    s = Side();
    cudaError_t e1 = cudaMalloc(&s.seq, total ? total : 1);
    cudaError_t e2 = e1 == cudaSuccess ? cudaMalloc(&s.offs, (n + 1) * sizeof(uint64_t)) : e1;
    cudaError_t e3 = e2 == cudaSuccess ? cudaMemcpy(s.seq, codes, total, cudaMemcpyHostToDevice) : e2;
    cudaError_t e4 = e3 == cudaSuccess ? cudaMemcpy(s.offs, offs, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice) : e3;
    std::free(codes);
    std::free(offs);
    if (e4 != cudaSuccess) {
        cudaFree(s.seq); cudaFree(s.offs); s = Side();
        return fail(e4 == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, "pg_set_seqs: %s", cudaGetErrorString(e4));
    }
    s.n = n;
    s.nres = total;
    s.maxlen = maxlen;
    ++c->epoch;
    return ensure_scratch(c);
}

int pg_share_row_seqs(pg_ctx *c)
{
    if (!c) return fail(PG_ERR_ARG, "null context");
    if (!c->side[0].seq) return fail(PG_ERR_STATE, "row sequences not set");
    CU(cudaSetDevice(c->cfg.device));
    if (!c->cols_share_rows) { cudaFree(c->side[1].seq); cudaFree(c->side[1].offs); }
    c->side[1] = c->side[0];
    c->cols_share_rows = true;
    ++c->epoch;
    return ensure_scratch(c);
}

// The traceback form of the DP phase: direction bytes per task, their
// offsets, then per chunk of consecutive tasks whose matrices fit the arena
// the DP kernel and the traceback kernel.  Reads the total size back to the
// host (one synchronization per batch, one more per extra chunk).
static int run_dir(pg_ctx *c, const pg::KParams &kp, uint64_t n, int grid, cudaStream_t st)
{
    const bool xdrop = c->cfg.mode == PG_MODE_XDROP;
    if (n + 1 > c->dirb_cap) {
        cudaFree(c->d_dbytes); cudaFree(c->d_doff); cudaFree(c->d_dsc); cudaFree(c->d_t1);
        cudaFree(c->d_scan);
        c->d_dbytes = nullptr; c->d_doff = nullptr; c->d_dsc = nullptr; c->d_t1 = nullptr;
        c->d_scan = nullptr; c->dirb_cap = 0; c->scan_bytes = 0;
        CU(cudaMalloc(&c->d_dbytes, (n + 1) * sizeof(uint64_t)));
        CU(cudaMalloc(&c->d_doff, (n + 1) * sizeof(uint64_t)));
        CU(cudaMalloc(&c->d_dsc, n * 4 * sizeof(int)));
        CU(cudaMalloc(&c->d_t1, 2 * sizeof(uint64_t)));   // chunk end, checked regions
        CU(cub::DeviceScan::ExclusiveSum(nullptr, c->scan_bytes, c->d_dbytes, c->d_doff, n + 1));
        CU(cudaMalloc(&c->d_scan, c->scan_bytes));
        c->dirb_cap = n + 1;
    }
    const int gs = (int)std::min<uint64_t>((uint64_t)c->nsm * 8, (n + 256) / 256);
    unsigned long long *d_nchk = reinterpret_cast<unsigned long long *>(c->d_t1 + 1);
    CU(cudaMemsetAsync(d_nchk, 0, sizeof *d_nchk, st));
    pg::dir_sizes(xdrop, kp, c->d_dbytes, d_nchk, gs, st);
    size_t sb = c->scan_bytes;
    CU(cub::DeviceScan::ExclusiveSum(c->d_scan, sb, c->d_dbytes, c->d_doff, n + 1, st));
    uint64_t total = 0;
    unsigned long long nchk = 0;
    CU(cudaMemcpyAsync(&total, c->d_doff + n, sizeof total, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&nchk, d_nchk, sizeof nchk, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    const uint64_t budget = c->tune.dir_arena_mb > 0 ? ((uint64_t)c->tune.dir_arena_mb << 20) : c->dir_budget;
    if (c->dir_cap > budget) {           // a smaller cap than the arena held so far
        cudaFree(c->d_dir);
        c->d_dir = nullptr; c->dir_cap = 0;
    }
    // grow at least twofold (up to the cap): a stream of batches of growing
    // need reallocates a few times, not once per batch
    const uint64_t need = std::max<uint64_t>(16, std::min<uint64_t>(total, budget));
    const uint64_t want = need > c->dir_cap ? std::min<uint64_t>(budget, std::max<uint64_t>(need, 2 * c->dir_cap))
                                            : need;
    if (want > c->dir_cap) {
        cudaFree(c->d_dir);
        c->d_dir = nullptr; c->dir_cap = 0;
        CU(cudaMalloc(&c->d_dir, want));
        c->dir_cap = want;
    }
    const int dyn = kp.dir16_lim > 0 ? pg::DIR16_DYN_SMEM : pg::DP_DYN_SMEM;
    const int tie = c->cfg.tie;
    int launches = 1;
    uint64_t t0 = 0;
    while (t0 < n) {
        uint64_t t1 = n;
        if (total > c->dir_cap) {
            pg::dir_chunk_end(c->d_doff, t0, n, c->dir_cap, c->d_t1, st);
            uint64_t lim[3] = {0, 0, 0};
            CU(cudaMemcpyAsync(&lim[0], c->d_t1, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            t1 = lim[0];
            CU(cudaMemcpyAsync(&lim[1], c->d_doff + t0, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            CU(cudaMemcpyAsync(&lim[2], c->d_doff + t1, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            if (lim[2] - lim[1] > c->dir_cap) {          // one task larger than the arena
                cudaFree(c->d_dir);
                c->d_dir = nullptr; c->dir_cap = 0;
                CU(cudaMalloc(&c->d_dir, lim[2] - lim[1]));
                c->dir_cap = lim[2] - lim[1];
            }
            launches += 1;
        }
        CU(cudaMemsetAsync(c->d_counter + 3, 0, sizeof(unsigned int), st));
        const uint64_t nt = t1 - t0;
        const int g = (int)std::min<uint64_t>((uint64_t)grid, (nt + pg::WARPS - 1) / pg::WARPS);
        const int gt = (int)std::min<uint64_t>((uint64_t)c->nsm * 8, (nt + 255) / 256);
        launches += pg::dir_run(xdrop, tie, kp, t0, t1, c->d_doff, c->d_dir, c->d_dsc, g, dyn, gt, nchk > 0, st);
        CU(cudaGetLastError());
        t0 = t1;
    }
    return launches;   // k_dirsize, then per chunk (k_chunk_end,) the DP (and its checked pass) and the traceback
}

// The batch timing events.  Inside a stream capture they become external
// event-record nodes, so the host can still wait on them after a replay (a
// plain record node leaves an event the host cannot synchronize on).
static cudaError_t record_event(const pg_ctx *c, cudaEvent_t e, cudaStream_t st)
{
    return c->capturing ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal)
                        : cudaEventRecord(e, st);
}

static int launch(pg_ctx *c, const pg_pair *d_pairs, uint64_t n, uint64_t roff, uint64_t coff,
                  pg_result *d_out, cudaStream_t st)
{
    c->last_launches = 0;
    if (n == 0) return PG_OK;
    if (!c->side[0].seq || !c->side[1].seq) return fail(PG_ERR_STATE, "sequences not set");
    // work counters are 32-bit and run up to about n + chunk * warps
    if (n > 0x7fffffffull) return fail(PG_ERR_ARG, "batch of %llu pairs exceeds 2^31-1", (unsigned long long)n);
    pg::KParams kp;
    kp.pairs = d_pairs; kp.n = n; kp.roff = roff; kp.coff = coff;
    kp.rseq = c->side[0].seq; kp.roffs = c->side[0].offs; kp.nr = c->side[0].n;
    kp.cseq = c->side[1].seq; kp.coffs = c->side[1].offs; kp.nc = c->side[1].n;
    kp.out = d_out; kp.sm = c->d_sm;
    kp.go = c->go; kp.ge = c->ge; kp.xg = c->xg; kp.xdrop = c->cfg.xdrop;
    kp.seed_len = c->cfg.seed_len; kp.seed_count = c->cfg.seed_count; kp.flags = c->cfg.flags;
    kp.ani_thr = c->cfg.ani_thr; kp.cov_thr = c->cfg.cov_thr;
    int rc = ensure_batch(c, n);
    if (rc) return rc;
    kp.counter = c->d_counter; kp.status = c->d_status; kp.exec_cells = c->d_exec;
    kp.xd = c->d_xd; kp.ovf = c->d_ovf;
    kp.bnd = c->d_bnd; kp.bnd_bytes = c->bnd_bytes;
    kp.gring = c->d_gring; kp.gring_w = c->gring_w;
    kp.sched = c->d_counter + 4;
    kp.order = c->tune.bucket_order ? c->d_order : nullptr;
    kp.xsched = c->d_counter + 4 + pg::SCHED_WORDS;
    kp.rows_cap = c->tune.rows_max;
    kp.dir = c->tune.dp_traceback ? 1 : 0;
    kp.dir16_lim = c->tune.dp_traceback >= 2 ? c->lim16 : 0;
    kp.dir16_pair = c->tune.dp_traceback == 3 ? 1 : 0;
    // regions past dir16_lim run the checked 16-bit form while their borders fit:
    // local borders are 0, global ones go + (i - 1) * max(go, ge) >= -30000
    kp.dir16_side = 0;
    if (kp.dir16_lim > 0) {
        const int gmax = std::max(c->go, c->ge);
        if (c->cfg.mode == PG_MODE_SW || gmax >= 0) kp.dir16_side = 65535;
        else kp.dir16_side = std::min(65535, (pg::SAT16_DP - std::abs(c->go)) / -gmax);
    }
    CU(cudaMemsetAsync(c->d_counter, 0, (4 + pg::SCHED_WORDS + pg::XSCHED_WORDS) * sizeof(unsigned int), st));
    CU(cudaMemsetAsync(c->d_status, 0, sizeof(int), st));
    const uint64_t need_blocks = (n + pg::WARPS - 1) / pg::WARPS;
    uint64_t gmax = (uint64_t)c->grid;
    if (c->tune.dp_blocks_per_sm > 0)
        gmax = std::min<uint64_t>(gmax, (uint64_t)c->nsm * (uint64_t)c->tune.dp_blocks_per_sm);
    const int grid = (int)std::min<uint64_t>(gmax, need_blocks);
    const dim3 blk(pg::WARPS * 32);
    const int gsched = (int)std::min<uint64_t>((uint64_t)c->nsm * 8, (n + 255) / 256);
    CU(record_event(c, c->ev[0], st));
    if (c->cfg.mode == PG_MODE_XDROP) {
        // extension kernel: k_xdr (the band window in registers) where the gap
        // and X allow it; otherwise k_xdf (a direction per step, the next
        // task read ahead) while the resident sequences fit half of L2, k_xd
        // (each task run to its end, more resident warps) when residues
        // stream from DRAM
        const uint64_t nres = c->side[0].nres + (c->cols_share_rows ? 0 : c->side[1].nres);
        const bool reg_ok = pg::xdr_supported(kp.xg, c->cfg.xdrop);
        int form = c->tune.xd_stepped;
        if (form < 0) form = reg_ok ? 2 : (nres <= c->l2_bytes / 2 ? 1 : 0);
        if (form == 2 && !reg_ok) form = 1;
        const bool int16 = c->tune.xd_int16 && c->cfg.xdrop <= pg::XMAX16;
        const uint64_t need_xd = (2 * n + pg::XT - 1) / pg::XT;
        uint64_t xmax = (uint64_t)(int16 ? c->grid_xd_run
                                         : form == 2 ? c->grid_xdr : form == 1 ? c->grid_xd : c->grid_xd_run);
        if (c->tune.xd_blocks_per_sm > 0)
            xmax = std::min<uint64_t>(xmax, (uint64_t)c->nsm * (uint64_t)c->tune.xd_blocks_per_sm);
        const int gx = (int)std::min<uint64_t>(xmax, need_xd);
        const bool affine = (c->cfg.flags & PG_F_XDROP_AFFINE) != 0;
        int xlaunch = 0;
        if (affine) {
            // affine gaps: a warp per task, one launch, nothing overflows
            xlaunch = -1;
        } else if (!int16 && form == 2 && c->tune.bucket_order) {
            // the extension tasks longest length bound first
            pg::KParams ko = kp;
            ko.xorder = c->d_xorder;
            const int gord = (int)std::min<uint64_t>((uint64_t)c->nsm * 8, (n + 255) / 256);
            pg::k_xtask_hist<<<gord, 256, 0, st>>>(ko);
            pg::k_xtask_bucket<<<gord, 256, 0, st>>>(ko);
            kp.xorder = c->d_xorder;
            xlaunch = 2;
        }
        if (affine) {
            pg::k_xda<<<c->grid_wide, blk, 0, st>>>(kp);
        } else {
            if (int16) pg::k_xd16<<<gx, pg::XT, 0, st>>>(kp);
            else if (form == 2) pg::k_xdr<8><<<gx, pg::XT, 0, st>>>(kp);
            else if (form == 1) pg::k_xdf<<<gx, pg::XT, 0, st>>>(kp);
            else pg::k_xd<<<gx, pg::XT, 0, st>>>(kp);
            pg::k_xd_wide<<<c->grid_wide, blk, 0, st>>>(kp);
        }
        if (kp.order) {
            pg::k_hist<true><<<gsched, 256, 0, st>>>(kp);
            pg::k_bucket<true><<<gsched, 256, 0, st>>>(kp);
        }
        CU(record_event(c, c->ev[1], st));
        const int dyn = pg::DP_DYN_SMEM;
        if (kp.dir) {
            const int l = run_dir(c, kp, n, (int)gmax, st);
            if (l < 0) return l;
            c->last_launches = (kp.order ? 4 : 2) + l + xlaunch;
        } else {
            pg::stat_run(true, c->cfg.tie, kp, grid, dyn, st);
            c->last_launches = (kp.order ? 5 : 3) + xlaunch;
        }
    } else {
        if (kp.order) {
            pg::k_hist<false><<<gsched, 256, 0, st>>>(kp);
            pg::k_bucket<false><<<gsched, 256, 0, st>>>(kp);
        }
        CU(record_event(c, c->ev[1], st));
        const int dyn = pg::DP_DYN_SMEM;
        if (kp.dir) {
            const int l = run_dir(c, kp, n, (int)gmax, st);
            if (l < 0) return l;
            c->last_launches = (kp.order ? 2 : 0) + l;
        } else {
            pg::stat_run(false, c->cfg.tie, kp, grid, dyn, st);
            c->last_launches = kp.order ? 3 : 1;
        }
    }
    CU(record_event(c, c->ev[2], st));
    c->events_valid = true;
    CU(cudaGetLastError());
    return PG_OK;
}

// launch() directly, or through a CUDA graph captured once per batch shape
static int enqueue(pg_ctx *c, const pg_pair *d_pairs, uint64_t n, uint64_t roff, uint64_t coff,
                   pg_result *d_out, cudaStream_t st)
{
    // the traceback form reads sizes back to the host mid-batch: no capture
    if (!c->tune.graph || c->tune.dp_traceback || n == 0)
        return launch(c, d_pairs, n, roff, coff, d_out, st);
    if (!c->side[0].seq || !c->side[1].seq) return fail(PG_ERR_STATE, "sequences not set");
    int rc = ensure_batch(c, n);       // every allocation happens outside the capture
    if (rc) return rc;
    const pg_ctx::GraphKey key{d_pairs, d_out, n, roff, coff, c->epoch, st};
    if (!c->gexec || !(key == c->gkey)) {
        if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
        CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        rc = launch(c, d_pairs, n, roff, coff, d_out, st);
        c->capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return fail(PG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        const cudaError_t e2 = cudaGraphInstantiate(&c->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) { c->gexec = nullptr; return fail(PG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e2)); }
        c->gkey = key;
        c->graph_launches = c->last_launches;
    }
    CU(cudaGraphLaunch(c->gexec, st));
    c->last_launches = c->graph_launches;
    c->events_valid = true;
    return PG_OK;
}

static int check_status(pg_ctx *c)
{
    int st = 0;
    CU(cudaMemcpy(&st, c->d_status, sizeof st, cudaMemcpyDeviceToHost));
    if (st & pg::ST_BAD_INDEX) return fail(PG_ERR_ARG, "a pair refers to a sequence index out of range");
    if (st & pg::ST_BAD_SCHED) return fail(PG_ERR_CUDA, "internal: inconsistent bucket schedule");
    return PG_OK;
}

int pg_align_device(pg_ctx *c, const pg_pair *d_pairs, uint64_t n, uint64_t roff, uint64_t coff,
                    pg_result *d_out, void *stream)
{
    if (!c || (n > 0 && (!d_pairs || !d_out))) return fail(PG_ERR_ARG, "pg_align_device: bad argument");
    CU(cudaSetDevice(c->cfg.device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    return enqueue(c, d_pairs, n, roff, coff, d_out, st);
}

int pg_sync(pg_ctx *c)
{
    if (!c) return fail(PG_ERR_ARG, "null context");
    CU(cudaSetDevice(c->cfg.device));
    CU(cudaDeviceSynchronize());
    return check_status(c);
}

int pg_align(pg_ctx *c, const pg_pair *pairs, uint64_t n, uint64_t roff, uint64_t coff, pg_result *out)
{
    if (!c || (n > 0 && (!pairs || !out))) return fail(PG_ERR_ARG, "pg_align: bad argument");
    c->last_launches = 0;
    if (n == 0) return PG_OK;
    CU(cudaSetDevice(c->cfg.device));
    if (n > c->cap) {
        cudaFree(c->d_pairs); cudaFree(c->d_out);
        c->d_pairs = nullptr; c->d_out = nullptr; c->cap = 0;
        CU(cudaMalloc(&c->d_pairs, n * sizeof(pg_pair)));
        CU(cudaMalloc(&c->d_out, n * sizeof(pg_result)));
        c->cap = n;
    }
    CU(cudaMemcpyAsync(c->d_pairs, pairs, n * sizeof(pg_pair), cudaMemcpyHostToDevice, c->stream));
    int rc = enqueue(c, c->d_pairs, n, roff, coff, c->d_out, c->stream);
    if (rc) return rc;
    CU(cudaMemcpyAsync(out, c->d_out, n * sizeof(pg_result), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return check_status(c);
}

int pg_last_launches(const pg_ctx *c) { return c ? c->last_launches : 0; }

int pg_get_seqs(const pg_ctx *c, int32_t side, uint8_t *codes, uint64_t *offsets, uint64_t *n,
                uint64_t *total)
{
    if (!c || (side != 0 && side != 1)) return fail(PG_ERR_ARG, "pg_get_seqs: bad argument");
    const Side &s = c->side[side];
    if (!s.seq) return fail(PG_ERR_STATE, "sequences not set");
    CU(cudaSetDevice(c->cfg.device));
    uint64_t tot = 0;
    CU(cudaMemcpy(&tot, s.offs + s.n, sizeof tot, cudaMemcpyDeviceToHost));
    if (n) *n = s.n;
    if (total) *total = tot;
    if (offsets) CU(cudaMemcpy(offsets, s.offs, (s.n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (codes && tot) CU(cudaMemcpy(codes, s.seq, tot, cudaMemcpyDeviceToHost));
    return PG_OK;
}

void pg_tuning_default(pg_tuning *t)
{
    if (!t) return;
    std::memset(t, 0, sizeof *t);
    t->dp_blocks_per_sm = 0;
    t->xd_blocks_per_sm = 0;
    t->bucket_order = 1;
    t->rows_max = 8;
    t->graph = 0;
    t->xd_int16 = 0;
    t->dp_traceback = 0;
    t->dir_arena_mb = 0;
    t->xd_stepped = -1;
}

int pg_get_tuning(const pg_ctx *c, pg_tuning *out)
{
    if (!c || !out) return fail(PG_ERR_ARG, "pg_get_tuning: bad argument");
    *out = c->tune;
    return PG_OK;
}

int pg_set_tuning(pg_ctx *c, const pg_tuning *t)
{
    if (!c || !t) return fail(PG_ERR_ARG, "pg_set_tuning: bad argument");
    if (t->dp_blocks_per_sm < 0 || t->dp_blocks_per_sm > c->dp_per_sm)
        return fail(PG_ERR_ARG, "dp_blocks_per_sm %d outside 0..%d", t->dp_blocks_per_sm, c->dp_per_sm);
    if (t->xd_blocks_per_sm < 0 || t->xd_blocks_per_sm > 64)
        return fail(PG_ERR_ARG, "xd_blocks_per_sm %d outside 0..64", t->xd_blocks_per_sm);
    if (t->bucket_order != 0 && t->bucket_order != 1) return fail(PG_ERR_ARG, "bucket_order must be 0 or 1");
    if (t->rows_max < 1 || t->rows_max > 8) return fail(PG_ERR_ARG, "rows_max %d outside 1..8", t->rows_max);
    if (t->graph != 0 && t->graph != 1) return fail(PG_ERR_ARG, "graph must be 0 or 1");
    if (t->xd_int16 != 0 && t->xd_int16 != 1) return fail(PG_ERR_ARG, "xd_int16 must be 0 or 1");
    if (t->dp_traceback < 0 || t->dp_traceback > 3) return fail(PG_ERR_ARG, "dp_traceback must be 0..3");
    if (t->dir_arena_mb < 0) return fail(PG_ERR_ARG, "dir_arena_mb must be >= 0");
    if (t->xd_stepped < -1 || t->xd_stepped > 2) return fail(PG_ERR_ARG, "xd_stepped must be -1, 0, 1 or 2");
    c->tune = *t;
    ++c->epoch;                         // launch shapes changed: recapture
    return PG_OK;
}

}  // extern "C"

// internal (not exported): the resident sequences of a context, for the pair
// filter in pg_filter.cu
int pg_internal_seqs(const pg_ctx *c, const uint8_t **rseq, const uint64_t **roffs, uint64_t *nr,
                     const uint8_t **cseq, const uint64_t **coffs, uint64_t *nc, int *device,
                     void **stream, int *mode)
{
    if (!c || !c->side[0].seq || !c->side[1].seq) return fail(PG_ERR_STATE, "sequences not set");
    *rseq = c->side[0].seq; *roffs = c->side[0].offs; *nr = c->side[0].n;
    *cseq = c->side[1].seq; *coffs = c->side[1].offs; *nc = c->side[1].n;
    *device = c->cfg.device; *stream = (void *)c->stream; *mode = c->cfg.mode;
    return PG_OK;
}

int pg_internal_fail(int code, const char *msg) { return fail(code, "%s", msg); }

// internal: the context's device and stream
int pg_internal_device(const pg_ctx *c, int *device, void **stream)
{
    if (!c) return fail(PG_ERR_ARG, "null context");
    *device = c->cfg.device;
    *stream = (void *)c->stream;
    return PG_OK;
}

// internal: make device arrays (cudaMalloc'd, now owned by the context) the
// sequences of one side, as pg_set_seqs would
int pg_internal_adopt_side(pg_ctx *c, int side, uint8_t *d_codes, uint64_t *d_offs, uint64_t n,
                           uint32_t maxlen)
{
    Side &s = c->side[side];
    if (side == 1 && c->cols_share_rows) { s = Side(); c->cols_share_rows = false; }
    if (side == 0 && c->cols_share_rows) { c->side[1] = Side(); c->cols_share_rows = false; }
    cudaFree(s.seq); cudaFree(s.offs);
    s = Side();
    s.seq = d_codes;
    s.offs = d_offs;
    s.n = n;
    s.maxlen = maxlen;
    if (n > 0) CU(cudaMemcpy(&s.nres, d_offs + n, sizeof s.nres, cudaMemcpyDeviceToHost));
    ++c->epoch;
    return ensure_scratch(c);
}

// internal: the context's substitution table on the device (25 x 25 int8)
int pg_internal_score(const pg_ctx *c, const int8_t **d_sm)
{
    if (!c || !c->d_sm) return fail(PG_ERR_STATE, "no context");
    *d_sm = c->d_sm;
    return PG_OK;
}

extern "C" {

}  // extern "C"

// ---------------------------------------------------------------- DPX peak
// Throughput of the DPX add-max instruction (__viaddmax_s32, max(a + b, c)) over
// every SM: 8 independent chains per thread, so the pipe, not latency, limits.
namespace {
template <int CHAINS>
__global__ void k_dpx_peak(int iters, int b, int *sink)
{
    int a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = threadIdx.x + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = __viaddmax_s32(a[k], b, a[(k + 1) % CHAINS]);
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s ^= a[k];
    if (s == 0x7fffffff) sink[blockIdx.x] = s;
}
}  // namespace

extern "C" {

int pg_dpx_peak(int device, double *ops_per_s)
{
    if (!ops_per_s) return fail(PG_ERR_ARG, "null output");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(PG_ERR_NODEV, "device %d", device);
    CU(cudaSetDevice(device));
    int nsm = 0;
    CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    const int threads = 1024, blocks = nsm * 2, iters = 4096;
    int *sink = nullptr;
    CU(cudaMalloc(&sink, blocks * sizeof(int)));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    k_dpx_peak<8><<<blocks, threads>>>(iters, -1, sink);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        k_dpx_peak<8><<<blocks, threads>>>(iters, -1, sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return fail(PG_ERR_CUDA, "dpx peak: %s", cudaGetErrorString(err));
    *ops_per_s = (double)threads * blocks * iters * 8 / (best * 1e-3);
    return PG_OK;
}

// cells computed by the kernels since the context was created
unsigned long long pg_exec_cells(pg_ctx *c)
{
    unsigned long long v[2] = {0, 0};
    if (pg_exec_cells_split(c, v) != PG_OK) return 0;
    return v[0] + v[1];
}

int pg_exec_cells_split(pg_ctx *c, unsigned long long out[2])
{
    if (!c || !out) return fail(PG_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->cfg.device));
    CU(cudaMemcpy(out, c->d_exec, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    return PG_OK;
}

int pg_kernel_ms(pg_ctx *c, float out[2])
{
    if (!c || !out) return fail(PG_ERR_ARG, "null argument");
    out[0] = out[1] = 0.0f;
    if (!c->events_valid) return PG_OK;
    CU(cudaSetDevice(c->cfg.device));
    CU(cudaEventSynchronize(c->ev[2]));
    CU(cudaEventElapsedTime(&out[0], c->ev[0], c->ev[1]));
    CU(cudaEventElapsedTime(&out[1], c->ev[1], c->ev[2]));
    return PG_OK;
}

}  // extern "C"

// ------------------------------------------------- no-allocation SW entry point
//
// For callers that may not allocate device memory at all: plugins embedded in
// a host framework that owns the device memory pool (its allocator must not be
// bypassed, and a cudaMalloc there can fail or serialise the whole device), and
// step loops that must not call the allocator between steps.  Instead of a
// context's cudaMalloc'd scratch, the local-alignment kernel below keeps its
// work counter, status word, score table and per-warp DP rows in one
// file-scope device array of fixed size.  Every GPU that loads the library
// holds that array until the process exits.  The kernel is the
// statistics-carrying SW form (k_sw's recurrence), which needs no direction
// arena: about 2.5 times the DP time of pg_align's default traceback form.
namespace {

constexpr size_t kNoAllocBytes = (size_t)32 << 20;   // PG_NOALLOC_SCRATCH_BYTES
constexpr size_t kNoAllocHeader = 4096;              // counters, status, score table
constexpr int kMaxDevices = 64;
// byte offsets inside the array's header
constexpr size_t kNaCounters = 0;     // [0, 16): the work-queue counters
constexpr size_t kNaStatus = 16;      // [16, 20): status word (ST_* bits)
constexpr size_t kNaExec = 24;        // [24, 40): executed cells (X-drop, DP)
constexpr size_t kNaCleared = 64;     // [0, 64) is zeroed by every call
constexpr size_t kNaTable = 64;       // [64, 64 + 625): the score table
// the work queue's counter is 32-bit: it must not wrap while warps still pop
constexpr uint64_t kNoAllocMaxPairs = (1ull << 31) - 1;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// device address of g_noalloc_scratch per device; filled by the first call on
// that device (the host-side name of the array is only a stand-in)
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// residue codes the caller passed: any code outside 0..24 sets ST_BAD_CODE
// (the DP indexes its score tables by code)
__global__ void k_noalloc_codes(const uint8_t *__restrict__ rseq, const uint64_t *__restrict__ roffs,
                                uint64_t nr, const uint8_t *__restrict__ cseq,
                                const uint64_t *__restrict__ coffs, uint64_t nc, int *status)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    const uint64_t rb = roffs[0], re = roffs[nr];
    for (uint64_t i = rb + t0; i < re; i += stride) bad |= rseq[i] >= PG_NRES;
    const uint64_t cb = coffs[0], ce = coffs[nc];
    for (uint64_t i = cb + t0; i < ce; i += stride) bad |= cseq[i] >= PG_NRES;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, pg::ST_BAD_CODE);
}

// k_sw with the per-pair column length checked against the rows it was given
template <int TIE>
__global__ void __launch_bounds__(pg::WARPS * 32) k_sw_noalloc(const pg::KParams kp, int max_cols)
{
    __shared__ int ssm[32 * 32];
    // bad residue codes: align nothing (the call reports PG_ERR_ARG)
    if (*(volatile int *)kp.status & pg::ST_BAD_CODE) return;
    pg::load_sm(ssm, kp.sm);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * pg::WARPS + (threadIdx.x >> 5);
    void *bnd = (char *)kp.bnd + gw * kp.bnd_bytes;
    uint2 *prof = pg::g_dyn_prof + (threadIdx.x >> 5) * (pg::NCODES * 32);
    unsigned long long exec = 0;
    uint64_t p;
    pg::WarpQueue q;
    while (q.pop(&kp.counter[0], kp.n, p)) {
        const pg_pair pr = kp.pairs[p];
        const uint8_t *V, *Hs;
        int m, n;
        pg_result o = pg::empty_result();
        if (!pg::pair_seqs(kp, pr, V, m, Hs, n)) {
            if (lane == 0) { atomicOr(kp.status, pg::ST_BAD_INDEX); kp.out[p] = o; }
            continue;
        }
        // decreasing offsets give negative lengths
        if (m < 0 || n < 0 || n > max_cols || m > 65535) {
            if (lane == 0) { atomicOr(kp.status, pg::ST_TOO_LONG); kp.out[p] = o; }
            continue;
        }
        exec += (unsigned long long)m * (unsigned long long)n;
        o.cells = pg::sat_u32((uint64_t)m * (uint64_t)n);
        int score = 0, have = 0, ei = 0, ej = 0, i0 = 0, j0 = 0;
        uint32_t M = 0, D = 0, G = 0;
        if (m <= pg::L1::MAXSIDE && n <= pg::L1::MAXSIDE) {
            const pg::DpOut<pg::L1> d = pg::dp_dispatch<pg::L1, TIE>(V, m, Hs, n, ssm, prof, kp.go, kp.ge, bnd);
            score = d.score; have = d.have; ei = d.ei; ej = d.ej;
            M = d.st.M(); D = d.st.D(); G = d.st.G(); i0 = d.st.i0(); j0 = d.st.j0();
        } else {
            const pg::DpOut<pg::L2> d = pg::dp_dispatch<pg::L2, TIE>(V, m, Hs, n, ssm, prof, kp.go, kp.ge, bnd);
            score = d.score; have = d.have; ei = d.ei; ej = d.ej;
            M = d.st.M(); D = d.st.D(); G = d.st.G(); i0 = d.st.i0(); j0 = d.st.j0();
        }
        if (have) {
            const uint32_t L = (uint32_t)((ei - i0) + (ej - j0)) - D;
            o.score = score;
            o.aln_len = L; o.matches = M; o.gap_opens = G;
            o.beg_v = (uint16_t)i0; o.end_v = (uint16_t)ei;
            o.beg_h = (uint16_t)j0; o.end_h = (uint16_t)ej;
            if (L > 0) { o.identity = pg::identity_of(M, L); o.flags = 0; }
        }
        pg::apply_filter(o, m, n, kp.cov_thr, kp.ani_thr);
        if (lane == 0) kp.out[p] = o;
    }
    if (lane == 0 && exec) atomicAdd(kp.exec_cells + 1, exec);
}

// restores the caller's current device on every return path
struct DeviceGuard {
    int prev = -1;
    DeviceGuard() { cudaGetDevice(&prev); }
    ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

}  // namespace

extern "C" int pg_align_sw_noalloc(const pg_config *cfg,
                                   const uint8_t *d_row_codes, const uint64_t *d_row_offsets, uint64_t nrows,
                                   const uint8_t *d_col_codes, const uint64_t *d_col_offsets, uint64_t ncols,
                                   uint32_t max_col_len, const pg_pair *d_pairs, uint64_t n,
                                   uint64_t bl_roffset, uint64_t bl_coffset, pg_result *d_out,
                                   void *stream)
{
    if (!cfg) return fail(PG_ERR_ARG, "pg_align_sw_noalloc: null config");
    int rc = validate(cfg);
    if (rc) return rc;
    if (cfg->mode != PG_MODE_SW) return fail(PG_ERR_ARG, "pg_align_sw_noalloc: mode must be PG_MODE_SW");
    if (n == 0) return PG_OK;
    if (!d_row_codes || !d_row_offsets || !d_col_codes || !d_col_offsets || !d_pairs || !d_out)
        return fail(PG_ERR_ARG, "pg_align_sw_noalloc: null buffer");
    if (n > kNoAllocMaxPairs)
        return fail(PG_ERR_ARG, "pg_align_sw_noalloc: more than 2^31-1 pairs in one call");
    if (max_col_len > 65535)
        return fail(PG_ERR_RANGE, "pg_align_sw_noalloc: max_col_len %u above 65535", max_col_len);
    const size_t per_warp = (((size_t)max_col_len + 1) * sizeof(pg::Edge<pg::L2>) + 255) & ~(size_t)255;
    const size_t rows_bytes = kNoAllocBytes - kNoAllocHeader;
    const size_t fit_warps = rows_bytes / per_warp;
    if (fit_warps < (size_t)pg::WARPS)
        return fail(PG_ERR_RANGE, "pg_align_sw_noalloc: columns of %u residues need %zu bytes of rows "
                    "per block, the fixed scratch holds %zu", max_col_len, per_warp * pg::WARPS, rows_bytes);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev ||
        cfg->device >= kMaxDevices)
        return fail(PG_ERR_NODEV, "pg_align_sw_noalloc: device %d", cfg->device);
    DeviceGuard guard;
    CU(cudaSetDevice(cfg->device));
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[cfg->device]) {
            void *ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return fail(PG_ERR_CUDA, "pg_align_sw_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            CU(cudaFuncSetAttribute(k_sw_noalloc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, pg::DP_DYN_SMEM));
            CU(cudaFuncSetAttribute(k_sw_noalloc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, pg::DP_DYN_SMEM));
            CU(cudaFuncSetAttribute(k_sw_noalloc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, pg::DP_DYN_SMEM));
            CU(cudaFuncSetAttribute(k_sw_noalloc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, pg::DP_DYN_SMEM));
            g_noalloc_ptr[cfg->device] = ptr;
        }
        base = (unsigned char *)g_noalloc_ptr[cfg->device];
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the header (counters, status, executed cells) starts at zero on every
    // call; the array keeps whatever the previous call left
    int8_t table[PG_NRES * PG_NRES];
    if (cfg->score_matrix) std::memcpy(table, cfg->score_matrix, sizeof table);
    else blosum62(table);
    CU(cudaMemsetAsync(base, 0, kNaCleared, st));
    CU(cudaMemcpyAsync(base + kNaTable, table, sizeof table, cudaMemcpyHostToDevice, st));
    pg::KParams kp;
    std::memset(&kp, 0, sizeof kp);
    kp.pairs = d_pairs; kp.n = n; kp.roff = bl_roffset; kp.coff = bl_coffset;
    kp.rseq = d_row_codes; kp.roffs = d_row_offsets; kp.nr = nrows;
    kp.cseq = d_col_codes; kp.coffs = d_col_offsets; kp.nc = ncols;
    kp.out = d_out; kp.sm = (const int8_t *)(base + kNaTable);
    if (cfg->gap_semantics == PG_GAPS_AS_CALLED) { kp.go = cfg->gap_ext; kp.ge = cfg->gap_open; }
    else { kp.go = cfg->gap_open; kp.ge = cfg->gap_ext; }
    kp.xg = kp.ge; kp.xdrop = cfg->xdrop; kp.seed_len = cfg->seed_len;
    kp.seed_count = cfg->seed_count; kp.flags = cfg->flags;
    kp.ani_thr = cfg->ani_thr; kp.cov_thr = cfg->cov_thr;
    kp.counter = (unsigned int *)(base + kNaCounters);
    kp.status = (int *)(base + kNaStatus);
    kp.exec_cells = (unsigned long long *)(base + kNaExec);
    kp.bnd = base + kNoAllocHeader;
    kp.bnd_bytes = per_warp;
    int nsm = 0, per_sm = 0;
    CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg->device));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sw_noalloc<0>, pg::WARPS * 32, pg::DP_DYN_SMEM));
    uint64_t grid = (uint64_t)nsm * (uint64_t)std::max(per_sm, 1);
    grid = std::min<uint64_t>(grid, fit_warps / pg::WARPS);
    grid = std::min<uint64_t>(grid, (n + pg::WARPS - 1) / pg::WARPS);
    const dim3 blk(pg::WARPS * 32);
    const int dyn = pg::DP_DYN_SMEM;
    k_noalloc_codes<<<(unsigned)nsm * 4u, 256, 0, st>>>(d_row_codes, d_row_offsets, nrows, d_col_codes,
                                                       d_col_offsets, ncols, kp.status);
    switch (cfg->tie) {
    case 0: k_sw_noalloc<0><<<(unsigned)grid, blk, dyn, st>>>(kp, (int)max_col_len); break;
    case 1: k_sw_noalloc<1><<<(unsigned)grid, blk, dyn, st>>>(kp, (int)max_col_len); break;
    case 2: k_sw_noalloc<2><<<(unsigned)grid, blk, dyn, st>>>(kp, (int)max_col_len); break;
    default: k_sw_noalloc<3><<<(unsigned)grid, blk, dyn, st>>>(kp, (int)max_col_len); break;
    }
    CU(cudaGetLastError());
    int status = 0;
    CU(cudaMemcpyAsync(&status, base + kNaStatus, sizeof status, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (status & pg::ST_BAD_CODE)
        return fail(PG_ERR_ARG, "pg_align_sw_noalloc: a residue code outside 0..24 (nothing aligned)");
    if (status & pg::ST_BAD_INDEX)
        return fail(PG_ERR_ARG, "pg_align_sw_noalloc: a pair refers to a sequence index out of range");
    if (status & pg::ST_TOO_LONG)
        return fail(PG_ERR_RANGE, "pg_align_sw_noalloc: a column sequence is longer than max_col_len %u "
                    "or a row sequence longer than 65535", max_col_len);
    return PG_OK;
}
