/*
 * pastis_gb300.h -- C ABI of the GB300 batched pairwise aligner for PASTIS.
 *
 * Drop-in for the arithmetic behind PASTIS's aligner plug-in interface
 * (inc/align/PWAlign.hpp:20-82).  A PWAlign subclass on the host:
 *   construct_seqs / construct_seqs_bl (PWAlign.hpp:33-41)  -> pg_set_seqs
 *   aln_batch(tuples, beg, end, roff, coff, params)          -> pg_align
 *     replacing seqan::localAlignment      (src/align/SeqanFullAligner.cpp:231)
 *     and seqan::extendSeed + globalAlignment
 *                                         (src/align/SeqanXdropAligner.cpp:281-296)
 *     and computeAlignmentStats + the coverage/ANI filter
 *                                         (SeqanFullAligner.cpp:238-263,
 *                                          SeqanXdropAligner.cpp:303-354)
 * Plain C types only; no exceptions cross the ABI.  Every call returns 0 or a
 * negative PG_ERR_* code; pg_strerror names it and pg_last_error gives detail.
 * One context per host thread (a context is not thread-safe).
 */
#ifndef PASTIS_GB300_H
#define PASTIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes */
#define PG_OK            0
#define PG_ERR_ARG      -1   /* bad argument (null pointer, size, index, option) */
#define PG_ERR_CUDA     -2   /* a CUDA runtime call failed */
#define PG_ERR_OOM      -3   /* device or pinned-host allocation failed */
#define PG_ERR_STATE    -5   /* call order (e.g. pg_align before pg_set_seqs) */
#define PG_ERR_RANGE    -6   /* a size limit: sequence over 65535 residues, output capacity, product bound */
#define PG_ERR_NODEV    -7   /* no CUDA device / device id out of range */

/* ---- alignment modes (params_t::PwAln, inc/Types.hpp:52-59) */
#define PG_MODE_SW     0     /* --sfa: affine local alignment (ALN_SEQAN_FULL)  */
#define PG_MODE_XDROP  1     /* --sxa: seeded X-drop + global (ALN_SEQAN_XDROP) */

/* ---- how PASTIS's (gap_open, gap_ext) reach the score model.
 * PASTIS constructs seqan::Blosum62(gap_open, gap_ext)
 * (inc/align/SeqanFullAligner.hpp:35-38, SeqanXdropAligner.hpp:38-43); SeqAn's
 * two-argument Score constructor takes (gapExtend, gapOpen).  PG_GAPS_AS_CALLED
 * reproduces that (first gap position scores gap_ext, further positions
 * gap_open, X-drop uses gap_open); PG_GAPS_NOMINAL uses the parameters by name
 * (first position gap_open, further gap_ext, X-drop gap_ext). */
#define PG_GAPS_AS_CALLED 0
#define PG_GAPS_NOMINAL   1

/* ---- traceback tie-breaking (the choices SeqAn's traceback makes on ties) */
#define PG_TIE_H_E_BEFORE_F   1   /* H ties: diag > horizontal > vertical (default diag > vertical > horizontal) */
#define PG_TIE_GAP_OPEN_FIRST 2   /* gap ties: open > extend (default extend > open) */

/* ---- behaviour flags */
#define PG_F_SKIP_SPURIOUS_SEED 1 /* skip the (0,0) second seed of count==1 pairs
                                     (the reference extends it: SeqanXdropAligner.cpp:273-277) */
#define PG_F_XDROP_AFFINE       2 /* X-drop extension with affine gaps (first / further gap
                                     scores of the global alignment) instead of SeqAn's single
                                     gap score (SeqanXdropAligner.cpp:281-283); a warp per
                                     task, kept for a gap model that cannot be checked here */

/* ---- per-pair result flags */
#define PG_RF_EMPTY     1   /* no alignment columns (identity reported as 0) */
#define PG_RF_BAD_SEED  2   /* a seed ran past a sequence end and was clamped */
#define PG_RF_PASSED    4   /* coverage/ANI filter passed, score_aln = identity/100 */
#define PG_RF_FILTERED  8   /* pruned by the learned pair filter, not aligned */

#define PG_FILTER_FEATURES 16  /* k-mer overlap features per pair */

#define PG_NRES 25          /* residue codes, order ARNDCQEGHILKMFPSTWYVBZX*J */

typedef struct pg_config {
    int32_t mode;           /* PG_MODE_* */
    int32_t gap_open;       /* params_t::gap_open (default -11, src/main.cpp:158-161) */
    int32_t gap_ext;        /* params_t::gap_ext  (default -2,  src/main.cpp:163-166) */
    int32_t gap_semantics;  /* PG_GAPS_* */
    int32_t xdrop;          /* params_t::aln_seqan_xdrop (--sxa value) */
    int32_t seed_len;       /* params_t::klength (default 6) */
    int32_t seed_count;     /* params_t::seed_count (default 2) */
    int32_t tie;            /* PG_TIE_* */
    int32_t flags;          /* PG_F_* */
    int32_t ani_thr;        /* params_t::aln_ani_thr (30) */
    double  cov_thr;        /* params_t::aln_cov_thr (0.7) */
    int32_t device;         /* CUDA device ordinal */
    int32_t reserved;
    const int8_t *score_matrix; /* PG_NRES x PG_NRES row-major, or NULL for BLOSUM62 */
} pg_config;

/* One candidate pair = one tuple of pw_aln_batch (src/DistPWRunner.cpp:100-102):
 * local row / column index plus the CommonKmerLoc fields the aligner reads
 * (inc/Types.hpp:166-171): count, score, first = (rs0, cs0), second = (rs1, cs1). */
typedef struct pg_pair {
    uint32_t row, col;
    uint16_t rs0, cs0, rs1, cs1;
    uint16_t count;
    int16_t  score;
} pg_pair;

/* Per-pair result.  H = column sequence, V = row sequence; coordinates are
 * 0-based half-open residue ranges of the aligned region. */
typedef struct pg_result {
    int32_t  score;         /* SW: local score; X-drop: global score of the kept seed */
    uint32_t aln_len;       /* alignment columns */
    uint32_t matches;       /* identical columns */
    uint32_t gap_opens;     /* gap runs, counted per row */
    uint16_t beg_h, end_h, beg_v, end_v;
    float    identity;      /* (float)(100.0 * matches / aln_len) */
    float    score_aln;     /* identity/100 if the coverage/ANI filter passes, else 0 */
    uint8_t  seed_used;     /* X-drop: which seed was kept (0 or 1) */
    uint8_t  flags;         /* PG_RF_* */
    uint16_t pad;
    uint32_t cells;         /* algorithmic DP cells of this pair (saturating) */
} pg_result;

typedef struct pg_ctx pg_ctx;

/* Fill cfg with PASTIS's defaults for a mode (src/main.cpp:97-116, :153-176). */
void pg_config_default(pg_config *cfg, int32_t mode);

int  pg_create(const pg_config *cfg, pg_ctx **out);
void pg_destroy(pg_ctx *ctx);

/* Load the row (side 0) or column (side 1) sequences of this rank's block:
 * ASCII residues concatenated, offsets[0..n] (offsets[n] = total bytes).  Lower
 * case is folded, letters outside ARNDCQEGHILKMFPSTWYVBZX*J score as X.
 * Replaces construct_seqs / construct_seqs_bl (PWAlign.hpp:33-41). */
int pg_set_seqs(pg_ctx *ctx, int32_t side, const char *residues,
                const uint64_t *offsets, uint64_t n);
/* Use the row sequences for the columns too (diagonal grid cell,
 * SeqanFullAligner.cpp:82-87). */
int pg_share_row_seqs(pg_ctx *ctx);

/* Parse a FASTA buffer (host memory, len bytes) on the GPU straight into the
 * row (side 0) or column (side 1) sequences, as FastaData::FastaData parses a
 * block (src/FastaData.cpp:13-148): a record starts at the first '>' of a
 * line, newlines and '*' in sequence text are dropped, 'U'/'u' read as 'T',
 * and a record with fewer than k residues is removed where the reference
 * removes it.  *n_kept / *n_removed count records; orig_index (host, optional)
 * receives the record index of each kept sequence, up to orig_cap entries.
 * Replaces the host parse and construct_seqs in one step. */
int pg_set_seqs_fasta(pg_ctx *ctx, int32_t side, const char *fasta, uint64_t len, int32_t k,
                      uint64_t *n_kept, uint64_t *n_removed, uint64_t *orig_index,
                      uint64_t orig_cap);

/* Copy one side's resident sequences back (residue codes 0..24, offsets of
 * n+1 entries); NULL buffers skip the copy, so a first call can size them. */
int pg_get_seqs(const pg_ctx *ctx, int32_t side, uint8_t *codes, uint64_t *offsets,
                uint64_t *n, uint64_t *total);

/* Align n pairs in host memory; writes n results to host memory.  Pair i uses
 * row sequence pairs[i].row + bl_roffset and column sequence
 * pairs[i].col + bl_coffset (PWAlign::aln_batch, PWAlign.hpp:47-63).  n == 0
 * is a no-op.  Synchronous. */
int pg_align(pg_ctx *ctx, const pg_pair *pairs, uint64_t n,
             uint64_t bl_roffset, uint64_t bl_coffset, pg_result *out);

/* Same, on device buffers, enqueued on `stream` (a cudaStream_t, NULL = the
 * context's stream); returns after enqueueing.  Call pg_sync (or synchronize
 * the stream) before reading `out`. */
int pg_align_device(pg_ctx *ctx, const pg_pair *d_pairs, uint64_t n,
                    uint64_t bl_roffset, uint64_t bl_coffset, pg_result *d_out,
                    void *stream);
int pg_sync(pg_ctx *ctx);

/* Number of kernel launches made by the last pg_align / pg_align_device call
 * (with graph replay: the kernels of the replayed graph). */
int pg_last_launches(const pg_ctx *ctx);

/* ---- launch tuning (no reference counterpart: SeqAn has no launch shape).
 * Every setting changes only how the batch is scheduled on the GPU; results
 * are identical under all of them.  pastis_gb300/autotune.py picks them by
 * timing candidates on a sample of the caller's own batch. */
typedef struct pg_tuning {
    int32_t dp_blocks_per_sm;   /* k_ga / k_sw resident blocks per SM; 0 = occupancy limit */
    int32_t xd_blocks_per_sm;   /* X-drop extension resident blocks per SM; 0 = occupancy limit */
    int32_t bucket_order;       /* 1: pairs in DP-bucket order, tallest first; 0: input order */
    int32_t rows_max;           /* cap on DP rows per lane, 1..8 (wide statistics stop at 4) */
    int32_t graph;              /* 1: pg_align / pg_align_device capture the batch's launches
                                   into a CUDA graph once per batch shape (pairs and output
                                   pointers, n, offsets, stream) and replay it after that */
    int32_t xd_int16;           /* 1: X-drop extension in 16-bit lanes, two cells per
                                   instruction; an extension whose score passes 30000 is
                                   rerun in 32 bits (needs xdrop <= 30000) */
    int32_t dp_traceback;       /* 1: the alignment DP stores a 4-bit decision per cell in an
                                   HBM arena (up to a third of the device memory, in chunks
                                   beyond that) and a traceback pass counts the statistics;
                                   2: the same, with two cells per instruction on 16-bit
                                   lanes for every region whose scores provably fit 16 bits
                                   ((m + n + 4) * largest |score| <= 30000); larger regions
                                   whose borders fit run there checked and are redone on
                                   32-bit lanes if a value leaves [-30000, 30000]; 32-bit
                                   lanes for the rest; 3: form 2, with the 16-bit regions
                                   of up to 32 * rows_max rows two per warp, each on half
                                   of it; no graph capture in these forms */
    int32_t dir_arena_mb;       /* cap on that arena in MiB; 0 = a third of the device memory */
    int32_t xd_stepped;         /* X-drop extension kernel, a thread per (pair, seed):
                                   2 holds the band's 16-column window in registers and
                                   computes it branch-free with packed 16-bit operations
                                   (needs a linear X-drop gap of -1..-4096 and xdrop
                                   <= 8192, else 1 runs); 1 steps one extension direction
                                   at a time over a shared-memory ring and starts the next
                                   the moment one ends; 0 runs each task to its end over
                                   the ring (fewer registers, more resident warps);
                                   -1 picks 2 where it applies, else 1 while the resident
                                   sequences fit half of L2, else 0 */
} pg_tuning;                    /* 36 bytes */

/* The built-in tuning.  A new context starts from it with dp_traceback = 3
 * (measured fastest in both modes); with a score table whose magnitudes pass
 * 100 (no region fits 16 bits) it takes 1 for PG_MODE_SW and keeps 0 for
 * PG_MODE_XDROP. */
void pg_tuning_default(pg_tuning *t);
int  pg_get_tuning(const pg_ctx *ctx, pg_tuning *out);
/* PG_ERR_ARG on a value out of range. */
int  pg_set_tuning(pg_ctx *ctx, const pg_tuning *t);

/* DP cells the kernels actually computed since pg_create (synchronizing read).
 * Differs from the sum of pg_result::cells where the kernel skips a second
 * seed whose extension or alignment repeats the first one's. */
unsigned long long pg_exec_cells(pg_ctx *ctx);
/* The same split as out[0] = X-drop band cells, out[1] = alignment DP cells. */
int pg_exec_cells_split(pg_ctx *ctx, unsigned long long out[2]);

/* Device time of the last pg_align / pg_align_device call, measured with CUDA
 * events on its stream: out[0] = seed extension (X-drop kernels; 0 for SW),
 * out[1] = alignment with statistics.  Waits for that batch to finish. */
int pg_kernel_ms(pg_ctx *ctx, float out[2]);

/* ---- learned candidate-pair filter
 * A learned form of the k-mer prune of pw_aln_batch (count <= ckthr or
 * score <= mosthr drops a pair, src/DistPWRunner.cpp:48-54): a 16-64-64-1 ReLU
 * network over k-mer overlap features, BF16 weights on the tensor cores with
 * FP32 accumulation, trained by the library's own kernels. */
typedef struct pg_filter pg_filter;

int  pg_filter_create(int device, uint64_t seed, pg_filter **out);
void pg_filter_destroy(pg_filter *f);
int  pg_filter_nparams(void);
/* copy the FP32 parameters out (get != 0) or in (get == 0) */
int  pg_filter_params(pg_filter *f, float *host, int get);
/* PG_FILTER_FEATURES bf16 features per pair into d_features (n x 16);
 * waits for the stream */
int  pg_filter_features(pg_filter *f, pg_ctx *ctx, const pg_pair *d_pairs, uint64_t n,
                        uint64_t bl_roffset, uint64_t bl_coffset, void *d_features, void *stream);
/* logits (FP32) of n feature rows */
int  pg_filter_predict(pg_filter *f, const void *d_features, uint64_t n, float *d_logits, void *stream);
/* gradients of the mean weighted binary cross-entropy with logits; the host
 * buffer receives pg_filter_nparams() gradients followed by the loss */
int  pg_filter_gradients(pg_filter *f, const void *d_features, const float *d_labels,
                         const float *d_weights, uint64_t n, float *host_grad_and_loss, void *stream);
/* one Adam step (beta 0.9 / 0.999) on a mini-batch; *loss (optional) gets its loss */
int  pg_filter_train_step(pg_filter *f, const void *d_features, const float *d_labels,
                          const float *d_weights, uint64_t n, float lr, float *loss, void *stream);
/* Align only the pairs whose logit is >= threshold; the others get an empty
 * result flagged PG_RF_FILTERED (score_aln 0).  *kept receives the count. */
int  pg_align_filtered(pg_ctx *ctx, pg_filter *f, float threshold, const pg_pair *d_pairs, uint64_t n,
                       uint64_t bl_roffset, uint64_t bl_coffset, pg_result *d_out, void *stream,
                       uint64_t *kept);

/* Local alignment (--sfa semantics, cfg->mode must be PG_MODE_SW) for callers
 * that may not allocate device memory: plugins running inside a host framework
 * that owns the device memory pool (its allocator must not be bypassed, and a
 * cudaMalloc there can fail or stall other work on the device), and step loops
 * that must not call the allocator between steps.  No reference counterpart:
 * PASTIS itself never runs on a GPU.  Nothing is allocated; the caller passes
 * every input and output as device buffers (sequences as residue codes 0..24
 * in the order ARNDCQEGHILKMFPSTWYVBZX*J, offsets of nrows+1 / ncols+1
 * entries, pairs, results), and the kernel's scratch (work counter, status,
 * score table, one DP row per warp) lives in one fixed 32 MiB device array
 * that every GPU loading the library keeps until the process exits.  The
 * kernel is the statistics-carrying SW form, about 2.5 times the DP time of
 * pg_align's default traceback form, which needs an arena this array cannot
 * hold.  Limits: max_col_len bounds the column sequences (at most 65535; a
 * longer one gives PG_ERR_RANGE), rows are at most 65535 residues, and one
 * call takes at most 2^31 - 1 pairs.  Errors: PG_ERR_ARG for a residue code
 * outside 0..24 (nothing is aligned, d_out is left as it was) or a pair whose
 * sequence index is out of range (its result is the empty one), PG_ERR_RANGE
 * for a sequence over the limits (its result is the empty one).  The first
 * call on a device looks up the array's device address.  Every call clears
 * the counters and status it uses at its start; calls share the array, so two
 * calls that overlap on the GPU (other streams or threads) race: serialize
 * them.  The call synchronizes `stream` (NULL = the legacy default stream)
 * before it returns; results equal pg_align's bit for bit. */
int pg_align_sw_noalloc(const pg_config *cfg,
                        const uint8_t *d_row_codes, const uint64_t *d_row_offsets, uint64_t nrows,
                        const uint8_t *d_col_codes, const uint64_t *d_col_offsets, uint64_t ncols,
                        uint32_t max_col_len, const pg_pair *d_pairs, uint64_t n,
                        uint64_t bl_roffset, uint64_t bl_coffset, pg_result *d_out,
                        void *stream);

/* ---- candidate generation: the k-mer SpGEMM C = A·Aᵀ that feeds the aligner
 * (src/kmer/KmerOps.cpp:31-245 builds A, sim_search.cpp:154-157 multiplies,
 * inc/sr.hpp:30-117 is the KmerIntersectLoc semiring).  A holds one entry per
 * k-mer occurrence (code over the alphabet, offset, self score of the k-mer
 * over the alphabet's representative letters); C(r, c) gets
 *   count = occurrence pairs sharing a k-mer (16-bit, wrapping as ushort does),
 *   score = the largest shared k-mer self score,
 *   first  = (row offset, col offset) of the smallest (code, row off, col off),
 *   second = the same of the largest; (0, 0) when count == 1.
 * Pairs come out block-relative (row - row_begin, col - col_begin) in column-
 * major order (by col, then row), as PASTIS forms its tuples. */
#define PG_ALPH_PROTEIN   0   /* 25 letters ARNDCQEGHILKMFPSTWYVBZX*J       */
#define PG_ALPH_MURPHY10  1   /* murphy10 groups, 15 codes (inc/Alphabet.hpp:83-104) */

#define PG_PRUNE_NONE     0   /* keep every pair, the diagonal included           */
#define PG_PRUNE_EVEN_ODD 1   /* one of (r,c)/(c,r) by parity, r != c (sim_search.cpp:172-186) */
#define PG_PRUNE_UPPER    2   /* strict upper triangle r < c (sim_search.cpp:403-412) */

typedef struct pg_kmer_config {
    int32_t  k;              /* k-mer length (--kmer-len, default 6)             */
    int32_t  stride;         /* k-mer stride (--kmer-stride, default 1)          */
    int32_t  alphabet;       /* PG_ALPH_*                                        */
    int32_t  prune;          /* PG_PRUNE_*                                       */
    int32_t  ckthr;          /* drop pairs with count <= ckthr (0 keeps all)     */
    int32_t  mosthr;         /* drop pairs with score <= mosthr                  */
    uint64_t max_products;   /* occurrence pairs one call may hold; 0 = 2^31     */
} pg_kmer_config;            /* 32 bytes */

void pg_kmer_config_default(pg_kmer_config *kc);
/* Candidate pairs of rows [row_begin, row_end) x columns [col_begin, col_end)
 * of the context's row and column sequences into d_out (device, cap records).
 * *n_out = pairs found.  PG_ERR_RANGE when they exceed cap (d_out untouched,
 * *n_out = the count needed) or the occurrence pairs exceed max_products
 * (*n_out = 0); PG_ERR_ARG when alphabet_size^k exceeds 2^31 (the reference's
 * own limit) or a range is out of bounds.  Synchronous. */
int pg_candidates(pg_ctx *ctx, const pg_kmer_config *kc, uint64_t row_begin, uint64_t row_end,
                  uint64_t col_begin, uint64_t col_end, pg_pair *d_out, uint64_t cap,
                  uint64_t *n_out, void *stream);

/* The similarity-matrix triples of an aligned batch (src/sim_search.cpp:221-232
 * after the score_aln == 0 prune of src/DistPWRunner.cpp:149-153):
 * (row + bl_roffset, col + bl_coffset, score_aln) of every pair whose score_aln
 * is not 0, in batch order, into device arrays of n entries.  Synchronous. */
int pg_triples(const pg_pair *d_pairs, const pg_result *d_res, uint64_t n,
               uint64_t bl_roffset, uint64_t bl_coffset, uint64_t *d_rows, uint64_t *d_cols,
               float *d_vals, uint64_t *n_out, void *stream);

/* Measured throughput of the DPX add-max instruction on a device, in
 * instructions per second over all SMs (the roofline of the DP kernels). */
int pg_dpx_peak(int device, double *ops_per_s);

const char *pg_strerror(int code);
const char *pg_last_error(void);

/* Library version string and the device architecture it was compiled for. */
const char *pg_version(void);

#ifdef __cplusplus
}
#endif
#endif
