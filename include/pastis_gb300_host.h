/*
 * pastis_gb300_host.h -- C entry points of the C++ host side (libpastis_host.so):
 * the pw_aln_batch driver over the GPU aligner, and the Matrix Market writer
 * of the similarity matrix.  The C++ interface itself is
 * include/pastis_gb300_pwalign.hpp.
 */
#ifndef PASTIS_GB300_HOST_H
#define PASTIS_GB300_HOST_H

#include <stdint.h>

#include "pastis_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A caller-supplied aligner for pgh_pw_aln_batch: fills score_aln[0..n) for
 * pairs[0..n) (used to test the driver's pruning and batching without a GPU).
 * A nonzero return fails the batch: a negative value is returned as the
 * error code, a positive one as PG_ERR_STATE. */
typedef int (*pgh_align_cb)(const pg_pair *pairs, uint64_t n, uint64_t bl_roff, uint64_t bl_coff,
                            float *score_aln, void *user);

/* pw_aln_batch (src/DistPWRunner.cpp:25-165) over one rank's block of C given
 * as nnz triples (rows, cols, vals = CommonKmerLoc for PG_MODE_XDROP,
 * CommonKmerLight for PG_MODE_SW): ckthr / mosthr prune, batches of batch_sz,
 * alignment (the GPU aligner built from cfg, or cb when it is not NULL; cres
 * NULL = the columns are the rows), score_aln written through vals, then the
 * score_aln == 0 prune.  The surviving triples are written back to the front
 * of rows / cols / vals.  out_stats (5 entries): nnz in, after the k-mer
 * prune, after alignment, batches, empty batches given to cb; out_seconds
 * (4 entries): the aligner's align|pre, align|gpu, align|post and align
 * timers. */
int pgh_pw_aln_batch(int mode, const pg_config *cfg,
                     const char *rres, const uint64_t *roffs, uint64_t nr,
                     const char *cres, const uint64_t *coffs, uint64_t nc,
                     uint64_t nnz, uint64_t *rows, uint64_t *cols, void *vals,
                     uint64_t bl_roff, uint64_t bl_coff, uint64_t batch_sz, int ckthr, float mosthr,
                     pgh_align_cb cb, void *cb_user, uint64_t *out_stats, double *out_seconds);

/* Batch-level resume of pgh_pw_aln_batch (the --bsz loop of
 * src/DistPWRunner.cpp:118-132, batch count l_nnz / bsz + 1 at :85-87; the
 * reference itself has no resume).  The batches depend only on the nonzero
 * count after the k-mer prune and on batch_sz, so a run can start at any one:
 *   start_batch  in: batches before it count as aligned (their score_aln is in vals)
 *   next_batch   out: first batch not aligned
 *   last_end     out: end of the pair range of the last aligned batch
 *   complete     out: 1 when every batch is aligned and the score_aln == 0 prune ran
 * A run that stops early -- on_batch returned nonzero after a batch, or a batch
 * failed (the call then returns that batch's error code: a PG_ERR_* of the GPU
 * library, or the callback aligner's negative return value) -- writes back the
 * triples as the k-mer prune left them, with score_aln set for every batch
 * before next_batch, and skips the score_aln prune.  Calling again with those
 * triples and start_batch = next_batch finishes the stage with the result an
 * uninterrupted run gives. */
typedef struct pgh_batch_ctl {
    uint64_t start_batch;
    uint64_t next_batch;
    uint64_t last_end;
    int32_t  complete;
    int32_t  reserved;
} pgh_batch_ctl;

/* Called after each aligned batch; a nonzero return stops the run there. */
typedef int (*pgh_batch_cb)(uint64_t batch, uint64_t beg, uint64_t end, void *user);

/* pgh_pw_aln_batch with ctl (NULL: run every batch) and on_batch (may be NULL). */
int pgh_pw_aln_batch_resume(int mode, const pg_config *cfg,
                            const char *rres, const uint64_t *roffs, uint64_t nr,
                            const char *cres, const uint64_t *coffs, uint64_t nc,
                            uint64_t nnz, uint64_t *rows, uint64_t *cols, void *vals,
                            uint64_t bl_roff, uint64_t bl_coff, uint64_t batch_sz, int ckthr,
                            float mosthr, pgh_align_cb cb, void *cb_user, uint64_t *out_stats,
                            double *out_seconds, pgh_batch_ctl *ctl, pgh_batch_cb on_batch,
                            void *on_batch_user);

/* Write n similarity triples as a Matrix Market coordinate file (what PASTIS's
 * --align-file output holds, src/sim_search.cpp:268-269): header
 * "%%MatrixMarket matrix coordinate real general", then "nrows ncols n", then
 * one "row col value" line per triple with 1-based indices and the value in
 * the shortest decimal form that reads back to the same float. */
int pgh_write_mm(const char *path, uint64_t nrows, uint64_t ncols, const uint64_t *rows,
                 const uint64_t *cols, const float *vals, uint64_t n);

const char *pgh_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
