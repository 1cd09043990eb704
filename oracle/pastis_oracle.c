/*
 * pastis_oracle.c -- CPU oracle (test infrastructure; parity unpinned, see the header).
 *
 * Each function names the reference call site whose behaviour it restates.
 * Plain C99 + OpenMP, no ISA intrinsics: builds and gives identical integer
 * results on x86-64 and aarch64.
 */
#include "pastis_oracle.h"

#include <limits.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NEG (-(1 << 30))

/* ---------------------------------------------------------------- scoring */

/* Published BLOSUM62 (Henikoff & Henikoff 1992) in the order
 * A R N D C Q E G H I L K M F P S T W Y V B Z X *.  The reference's 25th letter J
 * (src/Alphabet.cpp:26) scores exactly like L there (inc/ScoreMat.hpp:104-131),
 * so it is derived from the L row below rather than tabulated. */
static const signed char B62_24[24][24] = {
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

void orc_blosum62(int8_t out[ORC_NRES * ORC_NRES])
{
    const int L = 10, J = 24;
    for (int a = 0; a < ORC_NRES; ++a)
        for (int b = 0; b < ORC_NRES; ++b) {
            int aa = (a == J) ? L : a, bb = (b == J) ? L : b;
            out[a * ORC_NRES + b] = (int8_t)B62_24[aa][bb];
        }
}

uint8_t orc_encode(char c)
{
    static const char *letters = "ARNDCQEGHILKMFPSTWYVBZX*J";
    unsigned char u = (unsigned char)c;
    if (u >= 'a' && u <= 'z') u = (unsigned char)(u - 'a' + 'A');
    for (int i = 0; i < ORC_NRES; ++i)
        if ((unsigned char)letters[i] == u) return (uint8_t)i;
    return 22; /* X */
}

/* ------------------------------------------------- affine DP with statistics
 *
 * Restates SeqAn's localAlignment / globalAlignment + computeAlignmentStats as
 * PASTIS calls them (src/align/SeqanFullAligner.cpp:231 and :246,
 * src/align/SeqanXdropAligner.cpp:296 and :308-319).
 *
 * Cell (i, j) aligns V[i-1] with H[j-1].  E = best path ending in a horizontal
 * gap (consumes H, gap in V), F = vertical gap (consumes V), H = best overall.
 *   E(i,j) = max(E(i,j-1) + ext, H(i,j-1) + first)
 *   F(i,j) = max(F(i-1,j) + ext, H(i-1,j) + first)
 *   H(i,j) = max(H(i-1,j-1) + s(V[i-1], H[j-1]), F(i,j), E(i,j) [, 0 local])
 * Statistics travel with the predecessor a traceback would choose, so the values
 * at the end cell are those of the traced alignment: D = diagonal columns,
 * M = identical columns, G = gap runs counted per row as computeAlignmentStats
 * counts them (a gap opened right after a gap of the same orientation continues
 * the run), (bi, bj) = first aligned residue (local only).
 */
typedef struct { uint32_t m, d, g, bi, bj; } st_t;

enum { CH_DIAG = 0, CH_E = 1, CH_F = 2, CH_ZERO = 3 };

typedef struct { int h, e; st_t sh, se; unsigned char ch; } colcell;

static void dp_align(const uint8_t *v, int m, const uint8_t *h, int n,
                     const orc_params *p, int local, orc_aln *out)
{
    const int go = p->gap_first, ge = p->gap_ext;
    const int e_first = (p->tie & ORC_TIE_H_E_BEFORE_F) != 0;
    const int open_first = (p->tie & ORC_TIE_GAP_OPEN_FIRST) != 0;
    colcell *col = (colcell *)malloc(sizeof(colcell) * (size_t)(m + 1));

    /* column j = 0 */
    for (int i = 0; i <= m; ++i) {
        colcell *c = &col[i];
        memset(c, 0, sizeof(*c));
        c->e = NEG;
        if (local) {
            c->h = 0; c->ch = CH_ZERO; c->sh.bi = (uint32_t)i; c->sh.bj = 0;
        } else if (i == 0) {
            c->h = 0; c->ch = CH_DIAG;
        } else {
            /* F chain down column 0 (H(i,0) = F(i,0)) */
            const colcell *u = &col[i - 1];
            int f_ext = (i == 1) ? NEG + ge : u->h + ge; /* F(i-1,0) == H(i-1,0) for i-1 >= 1 */
            int f_opn = u->h + go;
            int pick_open = open_first ? (f_opn >= f_ext) : (f_opn > f_ext);
            st_t s = u->sh;
            if (pick_open && u->ch != CH_F) s.g += 1;
            c->h = pick_open ? f_opn : f_ext;
            c->sh = s; c->ch = CH_F;
        }
    }

    int best = 0, bi = 0, bj = 0, have_best = 0;
    st_t bst; memset(&bst, 0, sizeof bst);

    for (int j = 1; j <= n; ++j) {
        const uint8_t hj = h[j - 1];
        /* row 0 of this column */
        colcell diag = col[0];             /* (0, j-1) */
        {
            colcell *c = &col[0];
            if (local) {
                c->h = 0; c->e = NEG; c->ch = CH_ZERO;
                memset(&c->sh, 0, sizeof c->sh); c->sh.bi = 0; c->sh.bj = (uint32_t)j;
                memset(&c->se, 0, sizeof c->se);
            } else {
                int e_ext = c->e + ge, e_opn = c->h + go;
                int pick_open = open_first ? (e_opn >= e_ext) : (e_opn > e_ext);
                st_t s;
                if (pick_open) { s = c->sh; if (c->ch != CH_E) s.g += 1; }
                else s = c->se;
                c->e = pick_open ? e_opn : e_ext;
                c->se = s;
                c->h = c->e; c->sh = s; c->ch = CH_E;
            }
        }
        int f_up = NEG;            /* F(i-1, j) */
        st_t sf_up; memset(&sf_up, 0, sizeof sf_up);
        for (int i = 1; i <= m; ++i) {
            colcell *c = &col[i];          /* holds (i, j-1) on entry */
            const colcell *u = &col[i - 1]; /* (i-1, j), already updated */
            /* E from the left */
            int e_ext = c->e + ge, e_opn = c->h + go;
            int pe = open_first ? (e_opn >= e_ext) : (e_opn > e_ext);
            int e = pe ? e_opn : e_ext;
            st_t se;
            if (pe) { se = c->sh; if (c->ch != CH_E) se.g += 1; } else se = c->se;
            /* F from above */
            int f_ext = f_up + ge, f_opn = u->h + go;
            int pf = open_first ? (f_opn >= f_ext) : (f_opn > f_ext);
            int f = pf ? f_opn : f_ext;
            st_t sf;
            if (pf) { sf = u->sh; if (u->ch != CH_F) sf.g += 1; } else sf = sf_up;
            /* diagonal from (i-1, j-1) */
            const uint8_t vi = v[i - 1];
            int dg = diag.h + p->sm[vi * ORC_NRES + hj];
            st_t sd = diag.sh; sd.d += 1; sd.m += (vi == hj);

            int hv = dg; unsigned char ch = CH_DIAG; st_t sh = sd;
            if (e_first) {
                if (e > hv) { hv = e; ch = CH_E; sh = se; }
                if (f > hv) { hv = f; ch = CH_F; sh = sf; }
            } else {
                if (f > hv) { hv = f; ch = CH_F; sh = sf; }
                if (e > hv) { hv = e; ch = CH_E; sh = se; }
            }
            if (local && hv <= 0) {
                hv = 0; ch = CH_ZERO;
                memset(&sh, 0, sizeof sh); sh.bi = (uint32_t)i; sh.bj = (uint32_t)j;
            }
            diag = *c;                 /* (i, j-1) is the diagonal of (i+1, j) */
            c->h = hv; c->e = e; c->sh = sh; c->se = se; c->ch = ch;
            f_up = f; sf_up = sf;
            if (local && hv > best) { best = hv; bi = i; bj = j; bst = sh; have_best = 1; }
        }
    }

    memset(out, 0, sizeof(*out));
    uint32_t D, M, G;
    int i0, j0, i1, j1;
    if (local) {
        if (!have_best) {
            out->score = 0; out->flags = ORC_RF_EMPTY;
            free(col);
            return;
        }
        out->score = best;
        D = bst.d; M = bst.m; G = bst.g;
        i0 = (int)bst.bi; j0 = (int)bst.bj; i1 = bi; j1 = bj;
    } else {
        out->score = col[m].h;
        D = col[m].sh.d; M = col[m].sh.m; G = col[m].sh.g;
        i0 = 0; j0 = 0; i1 = m; j1 = n;
    }
    uint32_t L = (uint32_t)((i1 - i0) + (j1 - j0)) - D;
    out->aln_len = L; out->matches = M; out->gap_opens = G;
    out->beg_v = (uint16_t)i0; out->end_v = (uint16_t)i1;
    out->beg_h = (uint16_t)j0; out->end_h = (uint16_t)j1;
    if (L == 0) { out->identity = 0.0f; out->flags |= ORC_RF_EMPTY; }
    else out->identity = (float)((100.0 * (double)M) / (double)L);
    free(col);
}

/* The same DP with the per-row state in flat arrays and the statistics packed
 * (md = M | D << 16, g = gap runs, b = i0 | j0 << 16), used by the batch entry
 * points, which are also the timed CPU baseline.  Values and choices are those
 * of dp_align (tests/test_oracle.py checks both on random pairs under every
 * tie policy); only the bookkeeping differs. */
typedef struct {
    int *h, *e;
    uint32_t *shm, *shg, *shb, *sem, *seg, *seb;
    unsigned char *ch;
    int cap;
} fastbuf;

static void fastbuf_reserve(fastbuf *fb, int rows)
{
    if (rows <= fb->cap) return;
    free(fb->h); free(fb->e); free(fb->shm); free(fb->shg); free(fb->shb);
    free(fb->sem); free(fb->seg); free(fb->seb); free(fb->ch);
    fb->cap = rows + 64;
    size_t k = (size_t)fb->cap;
    fb->h = (int *)malloc(k * sizeof(int)); fb->e = (int *)malloc(k * sizeof(int));
    fb->shm = (uint32_t *)malloc(k * 4); fb->shg = (uint32_t *)malloc(k * 4);
    fb->shb = (uint32_t *)malloc(k * 4); fb->sem = (uint32_t *)malloc(k * 4);
    fb->seg = (uint32_t *)malloc(k * 4); fb->seb = (uint32_t *)malloc(k * 4);
    fb->ch = (unsigned char *)malloc(k);
}

static void fastbuf_free(fastbuf *fb)
{
    free(fb->h); free(fb->e); free(fb->shm); free(fb->shg); free(fb->shb);
    free(fb->sem); free(fb->seg); free(fb->seb); free(fb->ch);
    memset(fb, 0, sizeof *fb);
}

static void dp_align_fast(const uint8_t *v, int m, const uint8_t *hs, int n,
                          const orc_params *p, int local, fastbuf *fb, orc_aln *out)
{
    const int go = p->gap_first, ge = p->gap_ext;
    const int e_first = (p->tie & ORC_TIE_H_E_BEFORE_F) != 0;
    const int open_first = (p->tie & ORC_TIE_GAP_OPEN_FIRST) != 0;
    const int gmax = go > ge ? go : ge;
    memset(out, 0, sizeof(*out));
    if (m == 0 || n == 0) {
        if (local) { out->flags = ORC_RF_EMPTY; return; }
        if (m + n == 0) { out->flags = ORC_RF_EMPTY; return; }
        out->score = go + (m + n - 1) * gmax;
        out->aln_len = (uint32_t)(m + n); out->gap_opens = 1;
        out->end_v = (uint16_t)m; out->end_h = (uint16_t)n;
        out->identity = 0.0f;
        return;
    }
    fastbuf_reserve(fb, m + 1);
    int *H = fb->h, *E = fb->e;
    uint32_t *SHm = fb->shm, *SHg = fb->shg, *SHb = fb->shb;
    uint32_t *SEm = fb->sem, *SEg = fb->seg, *SEb = fb->seb;
    unsigned char *CH = fb->ch;
    /* column 0 */
    for (int i = 0; i <= m; ++i) {
        E[i] = NEG; SEm[i] = 0; SEg[i] = 0; SEb[i] = 0; SHm[i] = 0;
        if (local) { H[i] = 0; CH[i] = CH_ZERO; SHg[i] = 0; SHb[i] = (uint32_t)i; }
        else if (i == 0) { H[i] = 0; CH[i] = CH_DIAG; SHg[i] = 0; SHb[i] = 0; }
        else { H[i] = go + (i - 1) * gmax; CH[i] = CH_F; SHg[i] = 1; SHb[i] = 0; }
    }
    int best = 0, bi = 0, bj = 0, have = 0;
    uint32_t bm = 0, bg = 0, bb = 0;
    for (int j = 1; j <= n; ++j) {
        const int8_t *srow = p->sm + hs[j - 1];   /* column of the table: sm[v*25 + h] */
        const uint8_t hj = hs[j - 1];
        int dH = H[0];
        uint32_t dm = SHm[0], dgg = SHg[0], db = SHb[0];
        /* row 0 */
        if (local) {
            H[0] = 0; E[0] = NEG; CH[0] = CH_ZERO;
            SHm[0] = 0; SHg[0] = 0; SHb[0] = (uint32_t)j << 16;
        } else {
            const int ext = E[0] + ge, opn = H[0] + go;
            const int po = open_first ? (opn >= ext) : (opn > ext);
            uint32_t sm_ = po ? SHm[0] : SEm[0];
            uint32_t sg_ = po ? SHg[0] + (CH[0] != CH_E) : SEg[0];
            E[0] = po ? opn : ext;
            SEm[0] = sm_; SEg[0] = sg_; SEb[0] = 0;
            H[0] = E[0]; SHm[0] = sm_; SHg[0] = sg_; SHb[0] = 0; CH[0] = CH_E;
        }
        int fU = NEG;                    /* F(i-1, j) */
        uint32_t fm = 0, fg = 0, fb_ = 0;
        for (int i = 1; i <= m; ++i) {
            const uint8_t vi = v[i - 1];
            /* E from the left (i, j-1) */
            const int eext = E[i] + ge, eopn = H[i] + go;
            const int pe = open_first ? (eopn >= eext) : (eopn > eext);
            const int ev = pe ? eopn : eext;
            const uint32_t em = pe ? SHm[i] : SEm[i];
            const uint32_t eg = pe ? SHg[i] + (CH[i] != CH_E) : SEg[i];
            const uint32_t eb = pe ? SHb[i] : SEb[i];
            /* F from above (i-1, j): H[i-1] is already this column's */
            const int fext = fU + ge, fopn = H[i - 1] + go;
            const int pf = open_first ? (fopn >= fext) : (fopn > fext);
            const int fv = pf ? fopn : fext;
            const uint32_t nfm = pf ? SHm[i - 1] : fm;
            const uint32_t nfg = pf ? SHg[i - 1] + (CH[i - 1] != CH_F) : fg;
            const uint32_t nfb = pf ? SHb[i - 1] : fb_;
            /* diagonal (i-1, j-1) */
            const int dgv = dH + p->sm[vi * ORC_NRES + hj];
            const uint32_t sdm = dm + (1u << 16) + (uint32_t)(vi == hj);
            /* winner by priority, without branches: diag > F > E (or diag > E > F) */
            int takeF, takeE;
            if (e_first) {
                const int me = ev > dgv;
                takeF = fv > (me ? ev : dgv);
                takeE = me && !takeF;
            } else {
                const int mf = fv > dgv;
                takeE = ev > (mf ? fv : dgv);
                takeF = mf && !takeE;
            }
            int hv = takeF ? fv : (takeE ? ev : dgv);
            unsigned char ch = takeF ? CH_F : (takeE ? CH_E : CH_DIAG);
            uint32_t hm = takeF ? nfm : (takeE ? em : sdm);
            uint32_t hg = takeF ? nfg : (takeE ? eg : dgg);
            uint32_t hb = takeF ? nfb : (takeE ? eb : db);
            if (local) {
                const int z = hv <= 0;
                hv = z ? 0 : hv;
                ch = z ? CH_ZERO : ch;
                hm = z ? 0 : hm;
                hg = z ? 0 : hg;
                hb = z ? ((uint32_t)i | ((uint32_t)j << 16)) : hb;
            }
            dH = H[i]; dm = SHm[i]; dgg = SHg[i]; db = SHb[i];
            H[i] = hv; E[i] = ev; CH[i] = ch;
            SHm[i] = hm; SHg[i] = hg; SHb[i] = hb;
            SEm[i] = em; SEg[i] = eg; SEb[i] = eb;
            fU = fv; fm = nfm; fg = nfg; fb_ = nfb;
            if (local && hv > best) { best = hv; bi = i; bj = j; bm = hm; bg = hg; bb = hb; have = 1; }
        }
        (void)srow;
    }
    uint32_t D, M, G;
    int i0, j0, i1, j1;
    if (local) {
        if (!have) { out->flags = ORC_RF_EMPTY; return; }
        out->score = best;
        D = bm >> 16; M = bm & 0xffffu; G = bg;
        i0 = (int)(bb & 0xffffu); j0 = (int)(bb >> 16); i1 = bi; j1 = bj;
    } else {
        out->score = H[m];
        D = SHm[m] >> 16; M = SHm[m] & 0xffffu; G = SHg[m];
        i0 = 0; j0 = 0; i1 = m; j1 = n;
    }
    uint32_t L = (uint32_t)((i1 - i0) + (j1 - j0)) - D;
    out->aln_len = L; out->matches = M; out->gap_opens = G;
    out->beg_v = (uint16_t)i0; out->end_v = (uint16_t)i1;
    out->beg_h = (uint16_t)j0; out->end_h = (uint16_t)j1;
    if (L == 0) { out->identity = 0.0f; out->flags |= ORC_RF_EMPTY; }
    else out->identity = (float)((100.0 * (double)M) / (double)L);
}

void orc_local(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p, orc_aln *out)
{
    dp_align(v, m, h, n, p, 1, out);
    out->cells = (uint32_t)((uint64_t)m * (uint64_t)n > 0xffffffffu ? 0xffffffffu : (uint64_t)m * n);
}

void orc_global(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p, orc_aln *out)
{
    dp_align(v, m, h, n, p, 0, out);
    out->cells = (uint32_t)((uint64_t)m * (uint64_t)n > 0xffffffffu ? 0xffffffffu : (uint64_t)m * n);
}

/* ------------------------------------------------------------------ X-drop
 *
 * Restates seqan::extendSeed(seed, H, V, EXTEND_BOTH, score, x, GappedXDrop())
 * as called at src/align/SeqanXdropAligner.cpp:281-283 (H = column sequence,
 * V = row sequence).  One direction at a time, by anti-diagonals d = 2, 3, ...
 * of the (V-consumed = "col", H-consumed = "row") grid with linear gap g:
 *   T(c, r) = max(T(c-1, r) + g, T(c, r-1) + g, T(c-1, r-1) + s)
 * A cell whose value falls below best - X is dead (treated as minus infinity);
 * best is the maximum over all completed anti-diagonals.  The computed columns
 * of each anti-diagonal form a band [lo, hi) that is trimmed of dead cells at
 * both ends (looking at the current and the previous anti-diagonal), widened by
 * one to the right and clipped to the grid; the extension stops when the band
 * is empty.  (The border slot one past the last V residue is never alive.)  The end point is the far corner when it is alive, otherwise a
 * fixed probe of the previous anti-diagonal, otherwise the first maximum of the
 * anti-diagonal before that ("longest extension").  Border cells on the two
 * axes count as alive when d*g > best - X (d = 1: when g >= -X).
 */
typedef struct { int *v; int off, len; } adiag;   /* v indexed by column (full width) */

static int adiag_get(const adiag *a, int col) { return a->v[col]; }

/* hseq/vseq point at the first residue to consume; hstep/vstep = +1 or -1.
 * Returns band cells; *dv, *dh = residues consumed in V and H (0 if none). */
static uint64_t xdrop_dir(const uint8_t *vseq, int nv, int vstep,
                          const uint8_t *hseq, int nh, int hstep,
                          const orc_params *p, int *dv, int *dh)
{
    *dv = 0; *dh = 0;
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return 0;
    const int g = p->xdrop_gap, X = p->xdrop;
    const int UND = NEG;
    int *buf = (int *)malloc(sizeof(int) * 3 * (size_t)(cols + 1));
    for (int k = 0; k < 3 * (cols + 1); ++k) buf[k] = UND;
    adiag A[3] = {{buf, 0, 0}, {buf + (cols + 1), 0, 0}, {buf + 2 * (cols + 1), 0, 0}};
    adiag *a1 = &A[0], *a2 = &A[1], *a3 = &A[2];
    uint64_t cells = 0;

    /* d = 0 and d = 1 */
    a2->off = 0; a2->len = 1; a2->v[0] = 0;
    a3->off = 0; a3->len = 2;
    a3->v[0] = a3->v[1] = (-g > X) ? UND : g;
    int best = 0, d = 1, lo = 1, hi = 2;

    while (lo < hi) {
        ++d;
        adiag *t = a1; a1 = a2; a2 = a3; a3 = t;
        a3->off = lo - 1;
        a3->len = hi + 1 - a3->off;
        a3->v[a3->off] = UND;
        a3->v[hi] = UND;
        if ((long long)d * g > (long long)best - X) {
            if (a3->off == 0) a3->v[0] = d * g;
            if (d == hi && hi < cols) a3->v[hi] = d * g;
        }
        int dbest = d * g;
        const int thr = best - X;
        for (int c = lo; c < hi; ++c) {
            int r = d - c;
            int tmp = adiag_get(a2, c - 1);
            int t2 = adiag_get(a2, c);
            if (t2 > tmp) tmp = t2;
            tmp += g;
            const uint8_t vr = vseq[vstep * (c - 1)], hr = hseq[hstep * (r - 1)];
            int dg = adiag_get(a1, c - 1) + p->sm[vr * ORC_NRES + hr];
            if (dg > tmp) tmp = dg;
            if (tmp < thr) a3->v[c] = UND;
            else { a3->v[c] = tmp; if (tmp > dbest) dbest = tmp; }
        }
        cells += (uint64_t)(hi - lo);
        if (dbest > best) best = dbest;
        while (lo - a3->off < a3->len && a3->v[lo] == UND &&
               lo - a2->off - 1 < a2->len && a2->v[lo - 1] == UND)
            ++lo;
        while (hi - a3->off > 0 && a3->v[hi - 1] == UND && a2->v[hi - 1] == UND)
            --hi;
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
    }

    int lc = a3->off + a3->len - 2;
    int lr = d - lc;
    int ls = a3->v[lc];
    if (ls == UND) {
        if (a2->v[a2->off + a2->len - 2] != UND) {
            lc = a2->off + a2->len - 2; lr = d - 1 - lc; ls = a2->v[lc];
        } else if (a2->len > 2 && a2->v[a2->off + a2->len - 3] != UND) {
            lc = a2->off + a2->len - 3; lr = d - 1 - lc; ls = a2->v[lc];
        }
    }
    if (ls == UND) {
        for (int k = 0; k < a1->len; ++k) {
            int val = a1->v[a1->off + k];
            if (val > ls) { ls = val; lc = a1->off + k; lr = d - 2 - lc; }
        }
    }
    if (ls != UND) { *dv = lc; *dh = lr; }
    free(buf);
    return cells;
}

/* The affine gap model of the same extension (switch ORC_F_XDROP_AFFINE).
 * SeqAn's GappedXDrop extension takes a single gap score
 * (SeqanXdropAligner.cpp:281-283 passes the aligner's Score object, whose
 * scoreGap is the extend score); which model SeqAn applies cannot be run here,
 * so this form is the other one.  It is Gotoh's three-state recurrence over
 * the same anti-diagonals, a gap of length L scoring first + (L-1)*further as
 * in the full DP (gap_first / gap_ext):
 *   E(c, r) = max(T(c-1, r) + first, E(c-1, r) + further)    (V consumed)
 *   F(c, r) = max(T(c, r-1) + first, F(c, r-1) + further)    (H consumed)
 *   T(c, r) = max(T(c-1, r-1) + s, E(c, r), F(c, r))
 * A cell whose T falls below best - X is dead in all three states.  The border
 * cell of anti-diagonal d scores first + (d-1)*further (in T and in the gap
 * state along its axis); border liveness, band trimming and the end point are
 * those of the linear form with d*g replaced by that score.  With first ==
 * further == g both forms compute the same cells. */
static uint64_t xdrop_dir_affine(const uint8_t *vseq, int nv, int vstep,
                                 const uint8_t *hseq, int nh, int hstep,
                                 const orc_params *p, int *dv, int *dh)
{
    *dv = 0; *dh = 0;
    const int cols = nv + 1, rows = nh + 1;
    if (cols == 1 || rows == 1) return 0;
    const int go = p->gap_first, ge = p->gap_ext, X = p->xdrop;
    const int UND = NEG;
    const size_t W = (size_t)cols + 1;
    int *buf = (int *)malloc(sizeof(int) * 7 * W);
    for (size_t k = 0; k < 7 * W; ++k) buf[k] = UND;
    adiag A[3] = {{buf, 0, 0}, {buf + W, 0, 0}, {buf + 2 * W, 0, 0}};
    adiag *a1 = &A[0], *a2 = &A[1], *a3 = &A[2];
    int *E2 = buf + 3 * W, *E3 = buf + 4 * W, *F2 = buf + 5 * W, *F3 = buf + 6 * W;
    uint64_t cells = 0;

    /* d = 0: T(0,0) = 0; d = 1: the two border cells, T = first */
    a2->off = 0; a2->len = 1; a2->v[0] = 0;
    a3->off = 0; a3->len = 2;
    {
        const int v1 = (-go > X) ? UND : go;
        a3->v[0] = a3->v[1] = v1;
        F3[0] = v1;          /* (0, 1): a gap along H */
        E3[1] = v1;          /* (1, 0): a gap along V */
    }
    int best = 0, d = 1, lo = 1, hi = 2;

    while (lo < hi) {
        ++d;
        adiag *t = a1; a1 = a2; a2 = a3; a3 = t;
        int *te = E2; E2 = E3; E3 = te;
        int *tf = F2; F2 = F3; F3 = tf;
        a3->off = lo - 1;
        a3->len = hi + 1 - a3->off;
        a3->v[a3->off] = UND; E3[a3->off] = UND; F3[a3->off] = UND;
        a3->v[hi] = UND; E3[hi] = UND; F3[hi] = UND;
        const long long bscore = (long long)go + (long long)(d - 1) * ge;
        if (bscore > (long long)best - X) {
            if (a3->off == 0) { a3->v[0] = (int)bscore; F3[0] = (int)bscore; }
            if (d == hi && hi < cols) { a3->v[hi] = (int)bscore; E3[hi] = (int)bscore; }
        }
        int dbest = (int)(bscore < UND ? UND : bscore);
        const int thr = best - X;
        for (int c = lo; c < hi; ++c) {
            const int r = d - c;
            int e = a2->v[c - 1] + go;
            if (E2[c - 1] + ge > e) e = E2[c - 1] + ge;
            int f = a2->v[c] + go;
            if (F2[c] + ge > f) f = F2[c] + ge;
            const uint8_t vr = vseq[vstep * (c - 1)], hr = hseq[hstep * (r - 1)];
            int tmp = a1->v[c - 1] + p->sm[vr * ORC_NRES + hr];
            if (e > tmp) tmp = e;
            if (f > tmp) tmp = f;
            if (tmp < thr) { a3->v[c] = UND; E3[c] = UND; F3[c] = UND; }
            else {
                a3->v[c] = tmp; E3[c] = e; F3[c] = f;
                if (tmp > dbest) dbest = tmp;
            }
        }
        cells += (uint64_t)(hi - lo);
        if (dbest > best) best = dbest;
        while (lo - a3->off < a3->len && a3->v[lo] == UND &&
               lo - a2->off - 1 < a2->len && a2->v[lo - 1] == UND)
            ++lo;
        while (hi - a3->off > 0 && a3->v[hi - 1] == UND && a2->v[hi - 1] == UND)
            --hi;
        ++hi;
        if (lo < d + 2 - rows) lo = d + 2 - rows;
        if (hi > cols) hi = cols;
    }

    int lc = a3->off + a3->len - 2;
    int lr = d - lc;
    int ls = a3->v[lc];
    if (ls == UND) {
        if (a2->v[a2->off + a2->len - 2] != UND) {
            lc = a2->off + a2->len - 2; lr = d - 1 - lc; ls = a2->v[lc];
        } else if (a2->len > 2 && a2->v[a2->off + a2->len - 3] != UND) {
            lc = a2->off + a2->len - 3; lr = d - 1 - lc; ls = a2->v[lc];
        }
    }
    if (ls == UND) {
        for (int k = 0; k < a1->len; ++k) {
            int val = a1->v[a1->off + k];
            if (val > ls) { ls = val; lc = a1->off + k; lr = d - 2 - lc; }
        }
    }
    if (ls != UND) { *dv = lc; *dh = lr; }
    free(buf);
    return cells;
}

uint64_t orc_xdrop_extend(const uint8_t *v, int m, const uint8_t *h, int n,
                          const orc_params *p, int *bh, int *eh, int *bv, int *ev)
{
    int dv, dh;
    uint64_t cells = 0;
    uint64_t (*dir)(const uint8_t *, int, int, const uint8_t *, int, int, const orc_params *,
                    int *, int *) = (p->flags & ORC_F_XDROP_AFFINE) ? xdrop_dir_affine : xdrop_dir;
    /* left: prefixes V[0, bv), H[0, bh), consumed right to left */
    if (*bv > 0 && *bh > 0) {
        cells += dir(v + *bv - 1, *bv, -1, h + *bh - 1, *bh, -1, p, &dv, &dh);
        *bv -= dv; *bh -= dh;
    }
    /* right: suffixes V[ev, m), H[eh, n) */
    if (*ev < m && *eh < n) {
        cells += dir(v + *ev, m - *ev, +1, h + *eh, n - *eh, +1, p, &dv, &dh);
        *ev += dv; *eh += dh;
    }
    return cells;
}

/* ------------------------------------------------------- filter (a5 / a10) */

/* src/align/SeqanFullAligner.cpp:247-260 and SeqanXdropAligner.cpp:337-352:
 * keep iff max((L - G)/|c|, (L - G)/|r|) >= cov_thr and identity >= ani_thr,
 * then score_aln = identity / 100 (f32). */
static void apply_filter(orc_aln *o, int len_r, int len_c, const orc_params *p)
{
    double a = (double)o->aln_len - (double)o->gap_opens;
    double cc = a / (double)len_c, cr = a / (double)len_r;
    double cov = cc > cr ? cc : cr;
    if (!(o->flags & ORC_RF_EMPTY) && cov >= p->cov_thr && o->identity >= (float)p->ani_thr) {
        o->score_aln = o->identity / 100.0f;
        o->flags |= ORC_RF_PASSED;
    } else {
        o->score_aln = 0.0f;
    }
}

static uint32_t sat32(uint64_t x) { return x > 0xffffffffu ? 0xffffffffu : (uint32_t)x; }

void orc_sw_pair(const uint8_t *v, int m, const uint8_t *h, int n,
                 const orc_params *p, orc_aln *out)
{
    orc_local(v, m, h, n, p, out);
    out->seed_used = 0;
    apply_filter(out, m, n, p);
}

void orc_align_fast(const uint8_t *v, int m, const uint8_t *h, int n, const orc_params *p,
                    int local, orc_aln *out)
{
    fastbuf fb; memset(&fb, 0, sizeof fb);
    dp_align_fast(v, m, h, n, p, local, &fb, out);
    fastbuf_free(&fb);
    out->cells = sat32((uint64_t)m * (uint64_t)n);
}

static void sw_pair_fast(const uint8_t *v, int m, const uint8_t *h, int n,
                         const orc_params *p, fastbuf *fb, orc_aln *out)
{
    dp_align_fast(v, m, h, n, p, 1, fb, out);
    out->cells = sat32((uint64_t)m * (uint64_t)n);
    out->seed_used = 0;
    apply_filter(out, m, n, p);
}

/* src/align/SeqanXdropAligner.cpp:259-326: for each seed (first, second),
 * extend both ways, globally align the extended region, keep the strictly
 * higher identity; coverage uses the full sequence lengths (:340-341). */
static void xdrop_pair_impl(const uint8_t *v, int m, const uint8_t *h, int n,
                            const orc_pair *pr, const orc_params *p, fastbuf *fb, orc_aln *out);

void orc_xdrop_pair(const uint8_t *v, int m, const uint8_t *h, int n,
                    const orc_pair *pr, const orc_params *p, orc_aln *out)
{
    xdrop_pair_impl(v, m, h, n, pr, p, NULL, out);
}

/* fb == NULL: the plain DP (dp_align); otherwise the packed one */
static void xdrop_pair_impl(const uint8_t *v, int m, const uint8_t *h, int n,
                            const orc_pair *pr, const orc_params *p, fastbuf *fb, orc_aln *out)
{
    uint64_t cells = 0;
    int have = 0;
    orc_aln best; memset(&best, 0, sizeof best);
    best.flags = ORC_RF_EMPTY;
    int badseed = 0;
    for (int cnt = 0; cnt < p->seed_count && cnt < 2; ++cnt) {
        if (cnt > 0 && (p->flags & ORC_F_SKIP_SPURIOUS_SEED) && pr->count < 2) break;
        int r0 = cnt == 0 ? pr->rs0 : pr->rs1;
        int c0 = cnt == 0 ? pr->cs0 : pr->cs1;
        int bv = r0, ev = r0 + p->seed_len, bh = c0, eh = c0 + p->seed_len;
        if (ev > m || eh > n) {
            badseed = 1;
            if (bv > m) bv = m;
            if (ev > m) ev = m;
            if (bh > n) bh = n;
            if (eh > n) eh = n;
        }
        cells += orc_xdrop_extend(v, m, h, n, p, &bh, &eh, &bv, &ev);
        orc_aln cur;
        if (fb) dp_align_fast(v + bv, ev - bv, h + bh, eh - bh, p, 0, fb, &cur);
        else dp_align(v + bv, ev - bv, h + bh, eh - bh, p, 0, &cur);
        cells += (uint64_t)(ev - bv) * (uint64_t)(eh - bh);
        cur.beg_v = (uint16_t)bv; cur.end_v = (uint16_t)ev;
        cur.beg_h = (uint16_t)bh; cur.end_h = (uint16_t)eh;
        cur.seed_used = (uint8_t)cnt;
        /* an empty alignment has identity 0/0 = NaN in computeAlignmentStats:
         * it never replaces, and is never replaced by, a later seed */
        int cur_nan = (cur.flags & ORC_RF_EMPTY) != 0, best_nan = (best.flags & ORC_RF_EMPTY) != 0;
        if (!have || (!cur_nan && !best_nan && cur.identity > best.identity)) { best = cur; have = 1; }
    }
    *out = best;
    out->cells = sat32(cells);
    if (badseed) out->flags |= ORC_RF_BAD_SEED;
    apply_filter(out, m, n, p);
}

/* ----------------------------------------------------------------- batches */

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_batch(int mode,
              const uint8_t *rseq, const uint64_t *roffs, uint64_t nr,
              const uint8_t *cseq, const uint64_t *coffs, uint64_t nc,
              const orc_pair *pairs, uint64_t npairs,
              uint64_t bl_roff, uint64_t bl_coff,
              const orc_params *p, int nthreads, orc_aln *out)
{
    for (uint64_t i = 0; i < npairs; ++i)
        if (pairs[i].row + bl_roff >= nr || pairs[i].col + bl_coff >= nc) return -1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        fastbuf fb;
        memset(&fb, 0, sizeof fb);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (long long i = 0; i < (long long)npairs; ++i) {
            const orc_pair *pr = &pairs[i];
            uint64_t r = pr->row + bl_roff, c = pr->col + bl_coff;
            const uint8_t *v = rseq + roffs[r];
            const uint8_t *h = cseq + coffs[c];
            int m = (int)(roffs[r + 1] - roffs[r]);
            int n = (int)(coffs[c + 1] - coffs[c]);
            if (mode == 0) sw_pair_fast(v, m, h, n, p, &fb, &out[i]);
            else xdrop_pair_impl(v, m, h, n, pr, p, &fb, &out[i]);
        }
        fastbuf_free(&fb);
    }
    (void)nthreads;
    return 0;
}
