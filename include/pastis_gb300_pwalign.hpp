// pastis_gb300_pwalign.hpp -- C++ host side of the GB300 aligner, shaped like
// PASTIS's own aligner plug-in and batch driver so it drops into that code:
//
//   pastis::PWAlign                inc/align/PWAlign.hpp:20-82
//   pastis::GpuAligner : PWAlign   replaces SeqanFullAligner (--sfa,
//                                  src/align/SeqanFullAligner.cpp:173-266) and
//                                  SeqanXdropAligner (--sxa,
//                                  src/align/SeqanXdropAligner.cpp:190-361)
//   pastis::pw_aln_batch<NT>       src/DistPWRunner.cpp:25-165
//   CommonKmerLoc / CommonKmerLight / params_t   inc/Types.hpp:35-94, 163-266
//
// Differences forced by running without CombBLAS and MPI: the sequences come
// from a SeqSet (row / column sequences of this rank's block) instead of
// DistFastaData, and the rank's block of the candidate matrix is a LocalMat
// (column-major nonzeros, the order dcsc->cp / ir / jc walks them in
// DistPWRunner.cpp:96-105) instead of SpParMat.  Errors throw pastis::Error
// (a std::runtime_error with the PG_ERR_* code and pg_last_error()); there is
// no silent fallback.
#pragma once

#include <chrono>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "pastis_gb300.h"

namespace pastis {

typedef unsigned short ushort;

// inc/Types.hpp:163-215 (16 bytes)
struct CommonKmerLoc {
    ushort count;
    short score;
    float score_aln;
    std::pair<ushort, ushort> first;   // (row offset, column offset) of a shared k-mer
    std::pair<ushort, ushort> second;
    CommonKmerLoc() : count(1), score(-1), score_aln(0.0f), first(0, 0), second(0, 0) {}
    explicit CommonKmerLoc(ushort c) : count(c), score(-1), score_aln(0.0f), first(0, 0), second(0, 0) {}
};

// inc/Types.hpp:220-266 (8 bytes)
struct CommonKmerLight {
    ushort count;
    short score;
    float score_aln;
    CommonKmerLight() : count(1), score(-1), score_aln(0.0f) {}
    explicit CommonKmerLight(ushort c) : count(c), score(-1), score_aln(0.0f) {}
};

static_assert(sizeof(CommonKmerLoc) == 16, "CommonKmerLoc layout");
static_assert(sizeof(CommonKmerLight) == 8, "CommonKmerLight layout");

// the fields of params_t (inc/Types.hpp:35-94) this stage reads, with the
// defaults of src/main.cpp:97-116 and :153-176
struct params_t {
    enum PwAln { ALN_NONE = 0, ALN_SEQAN_FULL, ALN_SEQAN_XDROP, ALN_SEQAN_BANDED,
                 ALN_GPU_SW, ALN_GPU_XDROP };
    int gap_open = -11;
    int gap_ext = -2;
    ushort klength = 6;
    PwAln pw_aln = ALN_NONE;
    int aln_seqan_xdrop = 49;
    uint64_t aln_batch_sz = 10000000000ull;
    double aln_cov_thr = 0.7;
    int aln_ani_thr = 30;
    int seed_count = 2;
    int ckthr = 0;
    float mosthr = -1.0f;
};

// an error of the GPU library (or of an aligner's own call) with its code
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

// sequences of one side of the block: residues concatenated, offsets[n+1]
struct SeqSet {
    const char *residues = nullptr;
    std::vector<uint64_t> offsets;
    uint64_t size() const { return offsets.empty() ? 0 : offsets.size() - 1; }
};

// named wall-clock timers and counters, the ones TimePod keeps for this stage
// (inc/TraceUtils.hpp:31-71: align|pre, align|cpu, align|post, aln_pairs, ...)
struct StageTimers {
    std::map<std::string, double> seconds;
    std::map<std::string, double> counters;
    std::map<std::string, std::chrono::steady_clock::time_point> open;
    void start(const std::string &k) { open[k] = std::chrono::steady_clock::now(); }
    void stop(const std::string &k)
    {
        auto it = open.find(k);
        if (it == open.end()) return;
        seconds[k] += std::chrono::duration<double>(std::chrono::steady_clock::now() - it->second).count();
        open.erase(it);
    }
};

class PWAlign {
public:
    virtual ~PWAlign() {}
    virtual void construct_seqs(const SeqSet &rows, const SeqSet &cols) = 0;
    // diagonal grid cell: column sequences are the row sequences
    // (SeqanFullAligner.cpp:82-87)
    virtual void construct_seqs_bl(const SeqSet &rows) = 0;
    virtual void aln_batch(std::tuple<uint64_t, uint64_t, CommonKmerLight *> *mattuples,
                           uint64_t beg, uint64_t end, uint64_t bl_roffset, uint64_t bl_coffset,
                           const params_t &params) {}
    virtual void aln_batch(std::tuple<uint64_t, uint64_t, CommonKmerLoc *> *mattuples,
                           uint64_t beg, uint64_t end, uint64_t bl_roffset, uint64_t bl_coffset,
                           const params_t &params) {}
    virtual size_t rseq_len(uint64_t) { return 0; }
    virtual size_t cseq_len(uint64_t) { return 0; }
    StageTimers tp;
};

// The GPU aligner.  The two constructors mirror SeqanFullAligner(gap_open,
// gap_ext) and SeqanXdropAligner(gap_open, gap_ext, seed_len, xdrop, seed_cnt).
class GpuAligner : public PWAlign {
public:
    GpuAligner(int gap_open, int gap_ext, int device = 0,
               int gap_semantics = PG_GAPS_AS_CALLED, int tie = 0, int flags = 0)
    {
        pg_config c;
        pg_config_default(&c, PG_MODE_SW);
        c.gap_open = gap_open; c.gap_ext = gap_ext; c.device = device;
        c.gap_semantics = gap_semantics; c.tie = tie; c.flags = flags;
        init(c);
    }
    GpuAligner(int gap_open, int gap_ext, ushort seed_len, int xdrop, int seed_cnt,
               int device = 0, int gap_semantics = PG_GAPS_AS_CALLED, int tie = 0, int flags = 0)
    {
        pg_config c;
        pg_config_default(&c, PG_MODE_XDROP);
        c.gap_open = gap_open; c.gap_ext = gap_ext; c.seed_len = seed_len; c.xdrop = xdrop;
        c.seed_count = seed_cnt; c.device = device;
        c.gap_semantics = gap_semantics; c.tie = tie; c.flags = flags;
        init(c);
    }
    ~GpuAligner() override { pg_destroy(ctx_); }
    GpuAligner(const GpuAligner &) = delete;
    GpuAligner &operator=(const GpuAligner &) = delete;

    void construct_seqs(const SeqSet &rows, const SeqSet &cols) override
    {
        check(pg_set_seqs(ctx_, 0, rows.residues, rows.offsets.data(), rows.size()));
        check(pg_set_seqs(ctx_, 1, cols.residues, cols.offsets.data(), cols.size()));
        rlen_ = lengths(rows);
        clen_ = lengths(cols);
    }
    void construct_seqs_bl(const SeqSet &rows) override
    {
        check(pg_set_seqs(ctx_, 0, rows.residues, rows.offsets.data(), rows.size()));
        check(pg_share_row_seqs(ctx_));
        rlen_ = lengths(rows);
        clen_ = rlen_;
    }

    void aln_batch(std::tuple<uint64_t, uint64_t, CommonKmerLight *> *t, uint64_t beg, uint64_t end,
                   uint64_t bl_roffset, uint64_t bl_coffset, const params_t &params) override
    {
        run(t, beg, end, bl_roffset, bl_coffset, params);
    }
    void aln_batch(std::tuple<uint64_t, uint64_t, CommonKmerLoc *> *t, uint64_t beg, uint64_t end,
                   uint64_t bl_roffset, uint64_t bl_coffset, const params_t &params) override
    {
        run(t, beg, end, bl_roffset, bl_coffset, params);
    }
    size_t rseq_len(uint64_t i) override { return i < rlen_.size() ? rlen_[i] : 0; }
    size_t cseq_len(uint64_t i) override { return i < clen_.size() ? clen_[i] : 0; }

    // full per-pair results of the last batch (score, coordinates, statistics)
    const std::vector<pg_result> &last_results() const { return res_; }
    pg_ctx *context() { return ctx_; }

private:
    pg_ctx *ctx_ = nullptr;
    std::vector<pg_pair> pairs_;
    std::vector<pg_result> res_;
    std::vector<uint32_t> rlen_, clen_;

    static void check(int rc)
    {
        if (rc != PG_OK)
            throw Error(rc, std::string("pastis_gb300: ") + pg_strerror(rc) + ": " +
                                pg_last_error());
    }
    static std::vector<uint32_t> lengths(const SeqSet &s)
    {
        std::vector<uint32_t> l(s.size());
        for (uint64_t i = 0; i < s.size(); ++i) l[i] = (uint32_t)(s.offsets[i + 1] - s.offsets[i]);
        return l;
    }
    void init(const pg_config &c) { check(pg_create(&c, &ctx_)); }

    static void seeds(pg_pair &p, const CommonKmerLight *) { p.rs0 = p.cs0 = p.rs1 = p.cs1 = 0; }
    static void seeds(pg_pair &p, const CommonKmerLoc *v)
    {
        p.rs0 = v->first.first; p.cs0 = v->first.second;
        p.rs1 = v->second.first; p.cs1 = v->second.second;
    }

    template <typename NT>
    void run(std::tuple<uint64_t, uint64_t, NT *> *t, uint64_t beg, uint64_t end,
             uint64_t bl_roffset, uint64_t bl_coffset, const params_t &)
    {
        if (end <= beg) return;
        const uint64_t n = end - beg;
        tp.start("align|pre");
        pairs_.resize(n);
        res_.resize(n);
        double lens = 0;
        for (uint64_t i = 0; i < n; ++i) {
            const auto &tu = t[beg + i];
            const uint64_t r = std::get<0>(tu), c = std::get<1>(tu);
            if (r > 0xffffffffull || c > 0xffffffffull)
                throw Error(PG_ERR_ARG, "pastis_gb300: local index above 2^32");
            pg_pair &p = pairs_[i];
            p.row = (uint32_t)r; p.col = (uint32_t)c;
            p.count = std::get<2>(tu)->count;
            p.score = std::get<2>(tu)->score;
            seeds(p, std::get<2>(tu));
            lens += (double)rseq_len(r + bl_roffset) + (double)cseq_len(c + bl_coffset);
        }
        tp.counters["aln_pairs"] += (double)n;
        tp.counters["aln_pair_lens"] += lens;
        tp.stop("align|pre");
        tp.start("align|gpu");
        check(pg_align(ctx_, pairs_.data(), n, bl_roffset, bl_coffset, res_.data()));
        tp.stop("align|gpu");
        tp.start("align|post");
        // the reference writes score_aln only for pairs that pass; failing
        // entries are written as 0 so the post-prune sees them
        for (uint64_t i = 0; i < n; ++i) std::get<2>(t[beg + i])->score_aln = res_[i].score_aln;
        tp.stop("align|post");
    }
};

// The rank's block of the candidate matrix: nonzeros in column-major order.
template <typename NT>
struct LocalMat {
    std::vector<uint64_t> row, col;
    std::vector<NT> val;
    uint64_t nnz() const { return val.size(); }
    template <typename Pred>
    void prune(Pred drop)
    {
        uint64_t w = 0;
        for (uint64_t i = 0; i < val.size(); ++i) {
            if (drop(val[i])) continue;
            row[w] = row[i]; col[w] = col[i]; val[w] = val[i];
            ++w;
        }
        row.resize(w); col.resize(w); val.resize(w);
    }
};

struct BatchStats {
    uint64_t nnz_in = 0, nnz_kmer_thr = 0, nnz_aln = 0, batches = 0;
};

// Batch-level resume around the --bsz loop (src/DistPWRunner.cpp:118-132; the
// batch count l_nnz / bsz + 1 at :85-87).  The batch boundaries depend only on
// the pruned nonzero count and bsz, so a run can start at any batch:
//   start_batch  batches before it count as done (their score_aln is already in C)
//   on_batch     called after each aligned batch with its index and pair range;
//                returning false stops the run there (a job stopped between batches)
//   next_batch   out: the first batch not aligned (batch_cnt when all are)
//   last_end     out: end of the last aligned batch's pair range
//   complete     out: every batch aligned and the score_aln == 0 prune done
// A run that stops early, by on_batch or by an aligner error (which is then
// rethrown), leaves C as the k-mer prune left it, with score_aln written for
// every batch before next_batch, and does not run the score_aln prune.  Calling
// pw_aln_batch again on that C with start_batch = next_batch finishes the
// stage; the k-mer prune is idempotent, so the batches are the same.
struct BatchControl {
    uint64_t start_batch = 0;
    std::function<bool(uint64_t batch, uint64_t beg, uint64_t end)> on_batch;
    uint64_t next_batch = 0, last_end = 0;
    bool complete = false;
};

// src/DistPWRunner.cpp:25-165 on one rank's block: k-mer threshold prune,
// tuples, --bsz batches (batch_cnt = l_nnz / bsz + 1, so the trailing batch may
// be empty), then drop entries whose score_aln is 0.
template <typename NT>
BatchStats pw_aln_batch(LocalMat<NT> &C, PWAlign &pwa, const params_t &params,
                        uint64_t bl_roffset = 0, uint64_t bl_coffset = 0,
                        BatchControl *ctl = nullptr)
{
    BatchStats st;
    st.nnz_in = C.nnz();
    pwa.tp.start("prune");
    C.prune([&params](const NT &v) { return (v.count <= params.ckthr) || (v.score <= params.mosthr); });
    pwa.tp.stop("prune");
    st.nnz_kmer_thr = C.nnz();
    pwa.tp.start("align");
    const uint64_t l_nnz = C.nnz();
    bool stopped = false;
    if (l_nnz != 0) {
        const uint64_t bsz = params.aln_batch_sz ? params.aln_batch_sz : 1;
        const uint64_t batch_cnt = l_nnz / bsz + 1;
        const uint64_t b0 = ctl ? ctl->start_batch : 0;
        if (ctl) { ctl->next_batch = b0 < batch_cnt ? b0 : batch_cnt; ctl->last_end = 0; }
        pwa.tp.start("align|form-tuples");
        std::vector<std::tuple<uint64_t, uint64_t, NT *>> tuples(l_nnz);
        for (uint64_t k = 0; k < l_nnz; ++k) tuples[k] = std::make_tuple(C.row[k], C.col[k], &C.val[k]);
        pwa.tp.stop("align|form-tuples");
        pwa.tp.start("align|batch");
        for (uint64_t b = b0; b < batch_cnt; ++b) {
            const uint64_t beg = b * bsz;
            const uint64_t end = (b + 1) * bsz > l_nnz ? l_nnz : (b + 1) * bsz;
            try {
                pwa.aln_batch(tuples.data(), beg, end, bl_roffset, bl_coffset, params);
            } catch (...) {
                pwa.tp.stop("align|batch");
                pwa.tp.stop("align");
                throw;
            }
            ++st.batches;
            if (ctl) {
                ctl->next_batch = b + 1;
                ctl->last_end = end;
                if (ctl->on_batch && !ctl->on_batch(b, beg, end) && b + 1 < batch_cnt) {
                    stopped = true;
                    break;
                }
            }
        }
        pwa.tp.stop("align|batch");
    } else if (ctl) {
        ctl->next_batch = 0;
        ctl->last_end = 0;
    }
    pwa.tp.stop("align");
    if (stopped) {
        st.nnz_aln = C.nnz();
        return st;
    }
    pwa.tp.start("prune");
    C.prune([](const NT &v) { return v.score_aln == 0.0f; });
    pwa.tp.stop("prune");
    st.nnz_aln = C.nnz();
    if (ctl) ctl->complete = true;
    return st;
}

}  // namespace pastis
