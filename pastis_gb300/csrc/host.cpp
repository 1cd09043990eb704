// host.cpp -- C entry points over the C++ host side (pastis_gb300_pwalign.hpp),
// so that the batch driver can be exercised from any language.
//
// pgh_pw_aln_batch runs pw_aln_batch (src/DistPWRunner.cpp:25-165) on one
// rank's block with either the GPU aligner or a caller-supplied aligner
// callback (used to test the driver's pruning and batching without a GPU);
// pgh_pw_aln_batch_resume adds batch-level resume (pastis::BatchControl).
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>

#include "pastis_gb300.h"
#include "pastis_gb300_host.h"
#include "pastis_gb300_pwalign.hpp"

namespace {

thread_local std::string g_host_err;

class CallbackAligner : public pastis::PWAlign {
public:
    CallbackAligner(pgh_align_cb cb, void *user) : cb_(cb), user_(user) {}
    void construct_seqs(const pastis::SeqSet &, const pastis::SeqSet &) override {}
    void construct_seqs_bl(const pastis::SeqSet &) override {}
    void aln_batch(std::tuple<uint64_t, uint64_t, pastis::CommonKmerLight *> *t, uint64_t beg,
                   uint64_t end, uint64_t ro, uint64_t co, const pastis::params_t &) override
    {
        run(t, beg, end, ro, co);
    }
    void aln_batch(std::tuple<uint64_t, uint64_t, pastis::CommonKmerLoc *> *t, uint64_t beg,
                   uint64_t end, uint64_t ro, uint64_t co, const pastis::params_t &) override
    {
        run(t, beg, end, ro, co);
    }
    uint64_t calls = 0, empty_calls = 0;

private:
    pgh_align_cb cb_;
    void *user_;
    static void seeds(pg_pair &p, const pastis::CommonKmerLight *) { p.rs0 = p.cs0 = p.rs1 = p.cs1 = 0; }
    static void seeds(pg_pair &p, const pastis::CommonKmerLoc *v)
    {
        p.rs0 = v->first.first; p.cs0 = v->first.second;
        p.rs1 = v->second.first; p.cs1 = v->second.second;
    }
    template <typename NT>
    void run(std::tuple<uint64_t, uint64_t, NT *> *t, uint64_t beg, uint64_t end, uint64_t ro, uint64_t co)
    {
        ++calls;
        if (end <= beg) { ++empty_calls; return; }
        std::vector<pg_pair> p(end - beg);
        std::vector<float> s(end - beg, 0.0f);
        for (uint64_t i = beg; i < end; ++i) {
            pg_pair &q = p[i - beg];
            q.row = (uint32_t)std::get<0>(t[i]);
            q.col = (uint32_t)std::get<1>(t[i]);
            q.count = std::get<2>(t[i])->count;
            q.score = std::get<2>(t[i])->score;
            seeds(q, std::get<2>(t[i]));
        }
        const int rc = cb_(p.data(), end - beg, ro, co, s.data(), user_);
        if (rc != 0)
            throw pastis::Error(rc < 0 ? rc : PG_ERR_STATE, "aligner callback failed");
        for (uint64_t i = beg; i < end; ++i) std::get<2>(t[i])->score_aln = s[i - beg];
    }
};

template <typename NT>
int drive(int mode, const pg_config *cfg, const char *rres, const uint64_t *roffs, uint64_t nr,
          const char *cres, const uint64_t *coffs, uint64_t nc, uint64_t nnz, uint64_t *rows,
          uint64_t *cols, NT *vals, uint64_t bl_roff, uint64_t bl_coff, uint64_t batch_sz, int ckthr,
          float mosthr, pgh_align_cb cb, void *cb_user, uint64_t *out_stats, double *out_seconds,
          pgh_batch_ctl *ctl, pgh_batch_cb on_batch, void *on_batch_user)
{
    pastis::params_t params;
    params.aln_batch_sz = batch_sz;
    params.ckthr = ckthr;
    params.mosthr = mosthr;
    pastis::LocalMat<NT> C;
    C.row.assign(rows, rows + nnz);
    C.col.assign(cols, cols + nnz);
    C.val.assign(vals, vals + nnz);
    pastis::BatchStats st;
    std::unique_ptr<pastis::PWAlign> pwa;
    if (cb) {
        pwa.reset(new CallbackAligner(cb, cb_user));
    } else {
        if (!cfg) return PG_ERR_ARG;
        if (mode == PG_MODE_XDROP)
            pwa.reset(new pastis::GpuAligner(cfg->gap_open, cfg->gap_ext, (pastis::ushort)cfg->seed_len,
                                             cfg->xdrop, cfg->seed_count, cfg->device,
                                             cfg->gap_semantics, cfg->tie, cfg->flags));
        else
            pwa.reset(new pastis::GpuAligner(cfg->gap_open, cfg->gap_ext, cfg->device,
                                             cfg->gap_semantics, cfg->tie, cfg->flags));
        pastis::SeqSet R, Cs;
        R.residues = rres;
        R.offsets.assign(roffs, roffs + nr + 1);
        if (cres) {
            Cs.residues = cres;
            Cs.offsets.assign(coffs, coffs + nc + 1);
            pwa->construct_seqs(R, Cs);
        } else {
            pwa->construct_seqs_bl(R);
        }
    }
    pastis::BatchControl bc;
    if (ctl) {
        bc.start_batch = ctl->start_batch;
        if (on_batch)
            bc.on_batch = [on_batch, on_batch_user](uint64_t b, uint64_t beg, uint64_t end) {
                return on_batch(b, beg, end, on_batch_user) == 0;
            };
    }
    // a failed batch: what the earlier batches wrote stays in C, which goes
    // back to the caller with the error code
    int rc = PG_OK;
    st.nnz_in = nnz;
    try {
        st = pastis::pw_aln_batch(C, *pwa, params, bl_roff, bl_coff, ctl ? &bc : nullptr);
    } catch (const pastis::Error &e) {
        g_host_err = e.what();
        rc = e.code;
    }
    if (rc != PG_OK) {
        // the k-mer prune ran before the batch loop; nothing after it did
        st.nnz_kmer_thr = st.nnz_aln = C.nnz();
    }
    for (uint64_t i = 0; i < C.nnz(); ++i) { rows[i] = C.row[i]; cols[i] = C.col[i]; vals[i] = C.val[i]; }
    if (ctl) {
        ctl->next_batch = bc.next_batch;
        ctl->last_end = bc.last_end;
        ctl->complete = (rc == PG_OK && bc.complete) ? 1 : 0;
    }
    if (out_stats) {
        out_stats[0] = st.nnz_in; out_stats[1] = st.nnz_kmer_thr; out_stats[2] = st.nnz_aln;
        out_stats[3] = st.batches;
        CallbackAligner *ca = dynamic_cast<CallbackAligner *>(pwa.get());
        out_stats[4] = ca ? ca->empty_calls : 0;
    }
    if (out_seconds) {
        out_seconds[0] = pwa->tp.seconds["align|pre"];
        out_seconds[1] = pwa->tp.seconds["align|gpu"];
        out_seconds[2] = pwa->tp.seconds["align|post"];
        out_seconds[3] = pwa->tp.seconds["align"];
    }
    return rc;
}

}  // namespace

extern "C" int pgh_pw_aln_batch_resume(int mode, const pg_config *cfg,
                                       const char *rres, const uint64_t *roffs, uint64_t nr,
                                       const char *cres, const uint64_t *coffs, uint64_t nc,
                                       uint64_t nnz, uint64_t *rows, uint64_t *cols, void *vals,
                                       uint64_t bl_roff, uint64_t bl_coff, uint64_t batch_sz,
                                       int ckthr, float mosthr, pgh_align_cb cb, void *cb_user,
                                       uint64_t *out_stats, double *out_seconds,
                                       pgh_batch_ctl *ctl, pgh_batch_cb on_batch,
                                       void *on_batch_user)
{
    if (nnz && (!rows || !cols || !vals)) {
        g_host_err = "pgh_pw_aln_batch: null triple array";
        return PG_ERR_ARG;
    }
    try {
        if (mode == PG_MODE_XDROP)
            return drive(mode, cfg, rres, roffs, nr, cres, coffs, nc, nnz, rows, cols,
                         (pastis::CommonKmerLoc *)vals, bl_roff, bl_coff, batch_sz, ckthr, mosthr,
                         cb, cb_user, out_stats, out_seconds, ctl, on_batch, on_batch_user);
        if (mode == PG_MODE_SW)
            return drive(mode, cfg, rres, roffs, nr, cres, coffs, nc, nnz, rows, cols,
                         (pastis::CommonKmerLight *)vals, bl_roff, bl_coff, batch_sz, ckthr, mosthr,
                         cb, cb_user, out_stats, out_seconds, ctl, on_batch, on_batch_user);
        return PG_ERR_ARG;
    } catch (const pastis::Error &e) {
        g_host_err = e.what();
        return e.code;
    } catch (const std::exception &e) {
        g_host_err = e.what();
        return PG_ERR_STATE;
    }
}

extern "C" int pgh_pw_aln_batch(int mode, const pg_config *cfg,
                                const char *rres, const uint64_t *roffs, uint64_t nr,
                                const char *cres, const uint64_t *coffs, uint64_t nc,
                                uint64_t nnz, uint64_t *rows, uint64_t *cols, void *vals,
                                uint64_t bl_roff, uint64_t bl_coff, uint64_t batch_sz, int ckthr,
                                float mosthr, pgh_align_cb cb, void *cb_user, uint64_t *out_stats,
                                double *out_seconds)
{
    return pgh_pw_aln_batch_resume(mode, cfg, rres, roffs, nr, cres, coffs, nc, nnz, rows, cols,
                                   vals, bl_roff, bl_coff, batch_sz, ckthr, mosthr, cb, cb_user,
                                   out_stats, out_seconds, nullptr, nullptr, nullptr);
}

extern "C" int pgh_write_mm(const char *path, uint64_t nrows, uint64_t ncols, const uint64_t *rows,
                            const uint64_t *cols, const float *vals, uint64_t n)
{
    if (!path || (n && (!rows || !cols || !vals))) {
        g_host_err = "pgh_write_mm: bad argument";
        return PG_ERR_ARG;
    }
    FILE *f = std::fopen(path, "w");
    if (!f) {
        g_host_err = std::string("pgh_write_mm: cannot open ") + path;
        return PG_ERR_ARG;
    }
    std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n");
    std::fprintf(f, "%llu %llu %llu\n", (unsigned long long)nrows, (unsigned long long)ncols,
                 (unsigned long long)n);
    char buf[32];
    for (uint64_t i = 0; i < n; ++i) {
        if (rows[i] >= nrows || cols[i] >= ncols) {
            std::fclose(f);
            g_host_err = "pgh_write_mm: triple out of range";
            return PG_ERR_ARG;
        }
        // shortest %g form that reads back to the same float
        for (int prec = 6; prec <= 9; ++prec) {
            std::snprintf(buf, sizeof buf, "%.*g", prec, (double)vals[i]);
            if (std::strtof(buf, nullptr) == vals[i]) break;
        }
        std::fprintf(f, "%llu %llu %s\n", (unsigned long long)rows[i] + 1,
                     (unsigned long long)cols[i] + 1, buf);
    }
    const bool ok = std::fflush(f) == 0;
    std::fclose(f);
    if (!ok) {
        g_host_err = "pgh_write_mm: write failed";
        return PG_ERR_ARG;
    }
    return PG_OK;
}

extern "C" const char *pgh_last_error(void) { return g_host_err.c_str(); }
