/*
 * pastis_oracle.h -- CPU oracle for the batched pairwise-alignment stage of PASTIS.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark link it.  Nothing in the
 * product path (libpastis_gb300) calls it.
 *
 * PARITY UNPINNED.  The reference delegates every alignment to SeqAn
 * (src/align/SeqanFullAligner.cpp:231 localAlignment,
 *  src/align/SeqanXdropAligner.cpp:281-283 extendSeed(GappedXDrop),
 *  src/align/SeqanXdropAligner.cpp:296 globalAlignment,
 *  computeAlignmentStats at :246 / :308-319).  SeqAn is an empty, unpinned git
 * submodule in the reference checkout (.gitmodules:5-8, branch "develop"), so its
 * results cannot be reproduced here.  This file restates the published algorithms
 * (Gotoh 1982 affine local/global DP; X-drop extension, Zhang, Schwartz, Wagner &
 * Miller 2000) with every SeqAn convention that affects results made explicit:
 *
 *   - gap cost: a gap of length L scores gap_first + (L-1)*gap_ext (SeqAn's
 *     scoreGapOpen covers the first position of a gap);
 *   - which PASTIS parameter lands in which slot is decided by the caller
 *     (pg_scoring_from_params in the product library; the oracle takes the
 *     resolved numbers);
 *   - traceback tie-breaking (ORC_TIE_* bits), end-cell choice for local
 *     alignment (first maximum in column-major order: H index outer, V inner),
 *     alignment start at the last cell whose local score is <= 0;
 *   - X-drop: linear gap (SeqAn's GappedXDrop uses scoreGap == scoreGapExtend),
 *     anti-diagonal band with SeqAn's trimming and "longest extension" end rule,
 *     the anti-diagonal column axis is the V (row/query) sequence;
 *   - statistics as computeAlignmentStats reports them on the final alignment:
 *     alignment length = columns, gap opens = gap runs per row, identity =
 *     (float)(100.0 * matches / length).
 *
 * Residues are codes 0..24 in PASTIS's protein order ARNDCQEGHILKMFPSTWYVBZX*J
 * (src/Alphabet.cpp:26).
 */
#ifndef PASTIS_ORACLE_H
#define PASTIS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NRES 25

/* traceback tie-breaking */
#define ORC_TIE_H_E_BEFORE_F   1  /* H ties: diag > horizontal(E) > vertical(F); default diag > F > E */
#define ORC_TIE_GAP_OPEN_FIRST 2  /* E/F ties: open beats extend; default extend beats open */

/* behaviour switches */
#define ORC_F_SKIP_SPURIOUS_SEED 1 /* do not extend the second seed of a count==1 pair */
#define ORC_F_XDROP_AFFINE       2 /* X-drop with affine gaps (gap_first / gap_ext) */

/* result flags (same values as PG_RF_* in the product header) */
#define ORC_RF_EMPTY     1  /* alignment has no columns; identity reported as 0 */
#define ORC_RF_BAD_SEED  2  /* a seed ran past a sequence end and was clamped */
#define ORC_RF_PASSED    4  /* coverage/ANI filter passed (score_aln != 0) */

typedef struct orc_params {
    int32_t gap_first;   /* score of the first position of a gap (negative) */
    int32_t gap_ext;     /* score of every further position (negative) */
    int32_t xdrop_gap;   /* linear gap score used by X-drop extension */
    int32_t xdrop;       /* X-drop threshold */
    int32_t seed_len;    /* k-mer length (params.klength) */
    int32_t seed_count;  /* number of seeds tried (params.seed_count) */
    int32_t tie;         /* ORC_TIE_* */
    int32_t flags;       /* ORC_F_* */
    double  cov_thr;     /* params.aln_cov_thr */
    int32_t ani_thr;     /* params.aln_ani_thr */
    int8_t  sm[ORC_NRES * ORC_NRES]; /* substitution scores, row-major [a][b] */
} orc_params;

/* one candidate pair: local row / column sequence indices and the two seeds
 * (CommonKmerLoc::first / ::second, include/Types.hpp:170-171 of the reference) */
typedef struct orc_pair {
    uint32_t row, col;
    uint16_t rs0, cs0, rs1, cs1;
    uint16_t count;
    int16_t  score;
} orc_pair;

/* per-pair result; byte layout identical to pg_result */
typedef struct orc_aln {
    int32_t  score;
    uint32_t aln_len, matches, gap_opens;
    uint16_t beg_h, end_h, beg_v, end_v;
    float    identity, score_aln;
    uint8_t  seed_used, flags;
    uint16_t pad;
    uint32_t cells;      /* algorithmic DP cells for this pair (saturates at 2^32-1) */
} orc_aln;

/* the published BLOSUM62 matrix in PASTIS residue order */
void orc_blosum62(int8_t out[ORC_NRES * ORC_NRES]);
/* ASCII residue -> code (lower case folded, unknown letters -> X) */
uint8_t orc_encode(char c);

/* single alignments on code arrays; v = row/V sequence (length m), h = column/H (length n) */
void orc_local(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p, orc_aln *out);
void orc_global(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p, orc_aln *out);

/* The same DP as orc_local / orc_global with packed bookkeeping (what the batch
 * entry points use); local != 0 selects local alignment. */
void orc_align_fast(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p,
                    int local, orc_aln *out);

/* X-drop extension of one seed in both directions.  Seed = [*bh, *eh) x [*bv, *ev)
 * on entry and the extended region on exit.  Returns the number of band cells. */
uint64_t orc_xdrop_extend(const uint8_t *v, int m, const uint8_t *h, int n,
                          const orc_params *p, int *bh, int *eh, int *bv, int *ev);

/* one pair through the --sxa pipeline (all seeds, best identity, filter) */
void orc_xdrop_pair(const uint8_t *v, int m, const uint8_t *h, int n,
                    const orc_pair *pr, const orc_params *p, orc_aln *out);
/* one pair through the --sfa pipeline (local alignment, stats, filter) */
void orc_sw_pair(const uint8_t *v, int m, const uint8_t *h, int n,
                 const orc_params *p, orc_aln *out);

/* batches over packed sequences: codes concatenated, offsets[i]..offsets[i+1].
 * Pair i uses row sequence pairs[i].row + bl_roff and column sequence
 * pairs[i].col + bl_coff (the aln_batch contract).  nthreads <= 0: all cores.
 * mode 0 = SW (--sfa), 1 = X-drop (--sxa).  Returns 0, or -1 on a bad index. */
int orc_batch(int mode,
              const uint8_t *rseq, const uint64_t *roffs, uint64_t nr,
              const uint8_t *cseq, const uint64_t *coffs, uint64_t nc,
              const orc_pair *pairs, uint64_t npairs,
              uint64_t bl_roff, uint64_t bl_coff,
              const orc_params *p, int nthreads, orc_aln *out);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
