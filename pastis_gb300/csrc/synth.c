/*
 * synth.c -- seeded synthetic protein families and candidate pairs.
 *
 * Stands in for the reference's input (tests/scope_77k.fa is not shipped,
 * .MISSING_LARGE_BLOBS:1) and for its candidate producer (the k-mer SpGEMM,
 * src/kmer/KmerOps.cpp + inc/sr.hpp).  Every pair carries the fields of
 * CommonKmerLoc (inc/Types.hpp:163-215): a common k-mer count, the largest
 * k-mer self-score, and the offsets of the first and the last shared k-mer in
 * k-mer order (how KmerIntersectLoc::add folds them, inc/sr.hpp:67-78); a pair
 * with a single shared k-mer keeps the default (0, 0) second seed.
 *
 * Residues: 20 standard amino acids drawn at the BLOSUM62 background
 * frequencies (Henikoff & Henikoff 1992, as tabulated with the matrix by NCBI),
 * coded in PASTIS order ARNDCQEGHILKMFPSTWYVBZX*J.  Homologs: substitutions drawn
 * from P(b|a) proportional to p_b * 2^(S62(a,b)/2), b != a (the BLOSUM62
 * target-frequency ratio), then insertions/deletions of geometric length.
 *
 * Deterministic for a given seed: one xoshiro256** stream per family / pair.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/pastis_gb300_synth.h"

/* ------------------------------------------------------------- randomness */
static uint64_t splitmix64(uint64_t *x)
{
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

typedef struct { uint64_t s[4]; } rng_t;

static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(rng_t *r)
{
    uint64_t *s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return res;
}

static void rng_seed(rng_t *r, uint64_t seed, uint64_t stream)
{
    uint64_t x = seed ^ (stream * 0xd1342543de82ef95ULL);
    for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(&x);
}

static double rng_unif(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static uint32_t rng_u32(rng_t *r) { return (uint32_t)(rng_next(r) >> 32); }
static uint32_t rng_below(rng_t *r, uint32_t n) { return (uint32_t)(((uint64_t)rng_u32(r) * n) >> 32); }

static double rng_normal(rng_t *r)
{
    double u1 = rng_unif(r), u2 = rng_unif(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* geometric on {1, 2, ...} with the given mean */
static uint32_t rng_geom(rng_t *r, double mean)
{
    double p = 1.0 / mean;
    uint32_t k = 1;
    while (rng_unif(r) >= p && k < 1000) ++k;
    return k;
}

/* ------------------------------------------------------------- residues */

/* BLOSUM62 background frequencies, PASTIS order A R N D C Q E G H I L K M F P S T W Y V */
static const double BG[20] = {
    0.074, 0.052, 0.045, 0.053, 0.025, 0.034, 0.054, 0.074, 0.026, 0.068,
    0.099, 0.058, 0.025, 0.047, 0.039, 0.057, 0.051, 0.013, 0.032, 0.073};

/* BLOSUM62 among the 20 standard residues (same values as the aligner's table) */
static const signed char S20[20][20] = {
    { 4,-1,-2,-2, 0,-1,-1, 0,-2,-1,-1,-1,-1,-2,-1, 1, 0,-3,-2, 0},
    {-1, 5, 0,-2,-3, 1, 0,-2, 0,-3,-2, 2,-1,-3,-2,-1,-1,-3,-2,-3},
    {-2, 0, 6, 1,-3, 0, 0, 0, 1,-3,-3, 0,-2,-3,-2, 1, 0,-4,-2,-3},
    {-2,-2, 1, 6,-3, 0, 2,-1,-1,-3,-4,-1,-3,-3,-1, 0,-1,-4,-3,-3},
    { 0,-3,-3,-3, 9,-3,-4,-3,-3,-1,-1,-3,-1,-2,-3,-1,-1,-2,-2,-1},
    {-1, 1, 0, 0,-3, 5, 2,-2, 0,-3,-2, 1, 0,-3,-1, 0,-1,-2,-1,-2},
    {-1, 0, 0, 2,-4, 2, 5,-2, 0,-3,-3, 1,-2,-3,-1, 0,-1,-3,-2,-2},
    { 0,-2, 0,-1,-3,-2,-2, 6,-2,-4,-4,-2,-3,-3,-2, 0,-2,-2,-3,-3},
    {-2, 0, 1,-1,-3, 0, 0,-2, 8,-3,-3,-1,-2,-1,-2,-1,-2,-2, 2,-3},
    {-1,-3,-3,-3,-1,-3,-3,-4,-3, 4, 2,-3, 1, 0,-3,-2,-1,-3,-1, 3},
    {-1,-2,-3,-4,-1,-2,-3,-4,-3, 2, 4,-2, 2, 0,-3,-2,-1,-2,-1, 1},
    {-1, 2, 0,-1,-3, 1, 1,-2,-1,-3,-2, 5,-1,-3,-1, 0,-1,-3,-2,-2},
    {-1,-1,-2,-3,-1, 0,-2,-3,-2, 1, 2,-1, 5, 0,-2,-1,-1,-1,-1, 1},
    {-2,-3,-3,-3,-2,-3,-3,-3,-1, 0, 0,-3, 0, 6,-4,-2,-2, 1, 3,-1},
    {-1,-2,-2,-1,-3,-1,-1,-2,-2,-3,-3,-1,-2,-4, 7,-1,-1,-4,-3,-2},
    { 1,-1, 1, 0,-1, 0, 0, 0,-1,-2,-2, 0,-1,-2,-1, 4, 1,-3,-2,-2},
    { 0,-1, 0,-1,-1,-1,-1,-2,-2,-1,-1,-1,-1,-2,-1, 1, 5,-2,-2, 0},
    {-3,-3,-4,-4,-2,-2,-3,-2,-2,-3,-2,-3,-1, 1,-4,-3,-2,11, 2,-3},
    {-2,-2,-2,-3,-2,-1,-2,-3, 2,-1,-1,-2,-1, 3,-3,-2,-2, 2, 7,-1},
    { 0,-3,-3,-3,-1,-2,-2,-3,-3, 3, 1,-2, 1,-1,-2,-2, 0,-3,-1, 4}};

/* murphy10 groups of the reference (inc/Alphabet.hpp:83-104): DENQ->D, FWY->F,
 * ILMV->I, KR->K, ST->S; A C G H P stay. Value = representative's PASTIS code. */
static const uint8_t MURPHY10[20] = {
    /*A*/0, /*R*/11, /*N*/3, /*D*/3, /*C*/4, /*Q*/3, /*E*/3, /*G*/7, /*H*/8, /*I*/9,
    /*L*/9, /*K*/11, /*M*/9, /*F*/13, /*P*/14, /*S*/15, /*T*/15, /*W*/13, /*Y*/13, /*V*/9};

typedef struct {
    uint32_t bg_cum[20];       /* background thresholds (scaled to 2^32) */
    uint32_t sub_cum[20][20];  /* P(b | a), b != a */
} tables_t;

static void build_tables(tables_t *t)
{
    double sum = 0;
    for (int i = 0; i < 20; ++i) sum += BG[i];
    double acc = 0;
    for (int i = 0; i < 20; ++i) {
        acc += BG[i] / sum;
        t->bg_cum[i] = (i == 19) ? 0xffffffffu : (uint32_t)(acc * 4294967295.0);
    }
    for (int a = 0; a < 20; ++a) {
        double w[20], tot = 0;
        for (int b = 0; b < 20; ++b) {
            int s = S20[a][b];
            /* 2^(s/2) without libm: exact powers of two times sqrt(2) for odd s */
            double pw = (s % 2 == 0) ? ldexp(1.0, s / 2)
                                     : ldexp(1.4142135623730951, (s - 1) / 2);
            w[b] = (b == a) ? 0.0 : BG[b] * pw;
            tot += w[b];
        }
        double c = 0;
        for (int b = 0; b < 20; ++b) {
            c += w[b] / tot;
            t->sub_cum[a][b] = (b == 19 || (b == 18 && a == 19)) ? 0xffffffffu
                                                                : (uint32_t)(c * 4294967295.0);
        }
    }
}

static uint8_t draw_cum(rng_t *r, const uint32_t *cum)
{
    uint32_t u = rng_u32(r);
    int i = 0;
    while (i < 19 && u > cum[i]) ++i;
    return (uint8_t)i;
}

static uint32_t draw_len(rng_t *r, const pg_synth_cfg *c)
{
    double L;
    if (c->mix_frac > 0 && rng_unif(r) < c->mix_frac)
        L = c->mix_lo + rng_unif(r) * (double)(c->mix_hi - c->mix_lo);
    else
        L = c->len_median * exp(c->len_sigma * rng_normal(r));
    uint32_t l = (uint32_t)(L + 0.5);
    if (l < c->len_min) l = c->len_min;
    if (l > c->len_max) l = c->len_max;
    return l;
}

#define NOPOS 0xffffu

/* mutate src into dst (capacity cap) at target identity t; map[o] = the root
 * position residue o descends from (NOPOS for inserted residues); returns the
 * length */
static uint32_t mutate(rng_t *r, const tables_t *T, const uint8_t *src, uint32_t n,
                       double t, double indel_rate, double indel_mean,
                       uint8_t *dst, uint16_t *map, uint32_t cap, uint32_t min_len)
{
    uint32_t o = 0;
    for (uint32_t i = 0; i < n && o < cap; ++i) {
        if (indel_rate > 0 && rng_unif(r) < indel_rate) {
            uint32_t k = rng_geom(r, indel_mean);
            if (rng_u32(r) & 1u) {                 /* insertion before i */
                for (uint32_t q = 0; q < k && o < cap; ++q) {
                    map[o] = NOPOS;
                    dst[o++] = draw_cum(r, T->bg_cum);
                }
            } else {                               /* deletion of k residues */
                i += k - 1;
                continue;
            }
        }
        uint8_t a = src[i];
        if (o < cap) {
            map[o] = (uint16_t)(i < NOPOS ? i : NOPOS);
            dst[o++] = (rng_unif(r) < t) ? a : draw_cum(r, T->sub_cum[a]);
        }
    }
    while (o < min_len && o < cap) { map[o] = NOPOS; dst[o++] = draw_cum(r, T->bg_cum); }
    return o;
}

/* -------------------------------------------------------------- k-mers */

typedef struct { uint32_t code; uint16_t off; } kmer_t;

static int kmer_cmp(const void *a, const void *b)
{
    const kmer_t *x = (const kmer_t *)a, *y = (const kmer_t *)b;
    if (x->code != y->code) return x->code < y->code ? -1 : 1;
    return (int)x->off - (int)y->off;
}

/* distinct k-mers with their first offset, sorted by code */
static uint32_t kmers(const uint8_t *s, uint32_t n, uint32_t k, int alph, kmer_t *out)
{
    if (n < k) return 0;
    uint32_t cnt = 0;
    for (uint32_t i = 0; i + k <= n; ++i) {
        uint32_t code = 0;
        for (uint32_t q = 0; q < k; ++q) {
            uint8_t c = s[i + q];
            if (alph == 1 && c < 20) c = MURPHY10[c];
            code = code * 25u + c;
        }
        out[cnt].code = code; out[cnt].off = (uint16_t)(i > 65535 ? 65535 : i);
        ++cnt;
    }
    qsort(out, cnt, sizeof(kmer_t), kmer_cmp);
    uint32_t w = 0;
    for (uint32_t i = 0; i < cnt; ++i)
        if (w == 0 || out[w - 1].code != out[i].code) out[w++] = out[i];
    return w;
}

static int16_t self_score(const uint8_t *s, uint32_t k)
{
    int v = 0;
    for (uint32_t q = 0; q < k; ++q) { uint8_t c = s[q] < 20 ? s[q] : 0; v += S20[c][c]; }
    return (int16_t)v;
}

/* ------------------------------------------------------------- public */

struct pg_synth {
    uint8_t *seq; uint64_t *offs; uint64_t nseqs, nres;
    uint32_t *family;
    pg_pair *pairs; uint8_t *homolog, *spurious; uint64_t npairs;
};

static void seed_pair(const pg_synth_cfg *c, const uint8_t *rs, uint32_t m, const uint8_t *cs,
                      uint32_t n, rng_t *r, kmer_t *ka, kmer_t *kb, pg_pair *p, uint8_t *spurious,
                      const uint16_t *rmap, const uint16_t *cmap, uint32_t *inv)
{
    uint32_t na = kmers(rs, m, c->k, c->alph, ka), nb = kmers(cs, n, c->k, c->alph, kb);
    uint32_t i = 0, j = 0, count = 0;
    int16_t best = -1;
    uint16_t f0 = 0, f1 = 0, s0 = 0, s1 = 0;
    while (i < na && j < nb) {
        if (ka[i].code < kb[j].code) ++i;
        else if (ka[i].code > kb[j].code) ++j;
        else {
            if (count == 0) { f0 = ka[i].off; f1 = kb[j].off; }
            else { s0 = ka[i].off; s1 = kb[j].off; }
            int16_t sc = self_score(rs + ka[i].off, c->k);
            if (sc > best) best = sc;
            ++count; ++i; ++j;
        }
    }
    if (count == 0 && rmap && cmap) {
        /* homologs with no shared k-mer: one seed at offsets that descend from
         * the same root position (on the true alignment), as a seed found
         * through a reduced alphabet would be */
        uint32_t hits = 0;
        for (uint32_t q = 0; q + c->k <= n; ++q)
            if (cmap[q] != NOPOS && cmap[q] < 65535) inv[cmap[q]] = q + 1;
        for (uint32_t pp = 0; pp + c->k <= m; ++pp) {
            if (rmap[pp] == NOPOS || !inv[rmap[pp]]) continue;
            ++hits;
            if (rng_below(r, hits) == 0) { f0 = (uint16_t)pp; f1 = (uint16_t)(inv[rmap[pp]] - 1); }
        }
        for (uint32_t q = 0; q + c->k <= n; ++q)
            if (cmap[q] != NOPOS && cmap[q] < 65535) inv[cmap[q]] = 0;
        if (hits) {
            best = self_score(rs + f0, c->k);
            count = 1;
            *spurious = 2;
        }
    }
    if (count == 0) {
        /* no shared k-mer: one spurious seed at random valid offsets */
        f0 = (uint16_t)(m > c->k ? rng_below(r, m - c->k + 1) : 0);
        f1 = (uint16_t)(n > c->k ? rng_below(r, n - c->k + 1) : 0);
        best = self_score(rs + f0, m >= c->k ? c->k : m);
        count = 1;
        *spurious = 1;
    }
    p->count = (uint16_t)(count > 65535 ? 65535 : count);
    p->score = best;
    p->rs0 = f0; p->cs0 = f1;
    if (count >= 2) { p->rs1 = s0; p->cs1 = s1; } else { p->rs1 = 0; p->cs1 = 0; }
}

pg_synth *pg_synth_generate(const pg_synth_cfg *c)
{
    tables_t T;
    build_tables(&T);
    uint32_t fam_min = c->fam_min ? c->fam_min : 2, fam_max = c->fam_max >= fam_min ? c->fam_max : fam_min;
    /* family sizes */
    rng_t r0; rng_seed(&r0, c->seed, 0);
    uint64_t nfam = 0, total = 0;
    uint32_t *fsz = NULL; uint64_t cap = 0;
    while (total < c->nseqs) {
        uint32_t f = fam_min + (fam_max > fam_min ? rng_below(&r0, fam_max - fam_min + 1) : 0);
        if (total + f > c->nseqs) f = (uint32_t)(c->nseqs - total);
        if (nfam == cap) { cap = cap ? 2 * cap : 1024; fsz = (uint32_t *)realloc(fsz, cap * sizeof(uint32_t)); }
        fsz[nfam++] = f; total += f;
    }
    pg_synth *S = (pg_synth *)calloc(1, sizeof(pg_synth));
    S->nseqs = total;
    S->offs = (uint64_t *)malloc((total + 1) * sizeof(uint64_t));
    S->family = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
    uint64_t *fstart = (uint64_t *)malloc((nfam + 1) * sizeof(uint64_t));
    /* pass 1: root lengths bound member lengths; generate families into per-family buffers */
    uint8_t **fbuf = (uint8_t **)calloc(nfam ? nfam : 1, sizeof(uint8_t *));
    uint16_t **fmap = (uint16_t **)calloc(nfam ? nfam : 1, sizeof(uint16_t *));
    uint32_t **flen = (uint32_t **)calloc(nfam ? nfam : 1, sizeof(uint32_t *));
    uint64_t s = 0;
    for (uint64_t f = 0; f < nfam; ++f) { fstart[f] = s; s += fsz[f]; }
    fstart[nfam] = s;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long f = 0; f < (long long)nfam; ++f) {
        rng_t r; rng_seed(&r, c->seed, 1000003ULL + (uint64_t)f);
        uint32_t L = draw_len(&r, c);
        uint32_t capm = L * 2 + 64;
        if (capm > c->len_max + 64) capm = c->len_max + 64;
        if (capm < L) capm = L;
        uint8_t *buf = (uint8_t *)malloc((size_t)fsz[f] * capm);
        uint16_t *map = (uint16_t *)malloc((size_t)fsz[f] * capm * sizeof(uint16_t));
        uint32_t *ln = (uint32_t *)malloc(fsz[f] * sizeof(uint32_t));
        for (uint32_t q = 0; q < L; ++q) {
            buf[q] = draw_cum(&r, T.bg_cum);
            map[q] = (uint16_t)(q < NOPOS ? q : NOPOS);
        }
        ln[0] = L;
        for (uint32_t mbr = 1; mbr < fsz[f]; ++mbr) {
            double t = c->id_lo + rng_unif(&r) * (c->id_hi - c->id_lo);
            uint32_t mcap = capm < c->len_max ? capm : c->len_max;
            ln[mbr] = mutate(&r, &T, buf, L, t, c->indel_rate, c->indel_mean,
                             buf + (size_t)mbr * capm, map + (size_t)mbr * capm, mcap, c->len_min);
        }
        fbuf[f] = buf; fmap[f] = map; flen[f] = ln;
    }
    /* concatenate */
    uint64_t nres = 0;
    for (uint64_t f = 0; f < nfam; ++f)
        for (uint32_t mbr = 0; mbr < fsz[f]; ++mbr) nres += flen[f][mbr];
    S->nres = nres;
    S->seq = (uint8_t *)malloc(nres ? nres : 1);
    uint16_t *rootpos = (uint16_t *)malloc((nres ? nres : 1) * sizeof(uint16_t));
    uint64_t o = 0, si = 0;
    for (uint64_t f = 0; f < nfam; ++f) {
        uint32_t L0 = flen[f][0];
        uint32_t capm = L0 * 2 + 64;
        if (capm > c->len_max + 64) capm = c->len_max + 64;
        if (capm < L0) capm = L0;
        for (uint32_t mbr = 0; mbr < fsz[f]; ++mbr) {
            S->offs[si] = o;
            S->family[si] = (uint32_t)f;
            memcpy(S->seq + o, fbuf[f] + (size_t)mbr * capm, flen[f][mbr]);
            memcpy(rootpos + o, fmap[f] + (size_t)mbr * capm, flen[f][mbr] * sizeof(uint16_t));
            o += flen[f][mbr];
            ++si;
        }
        free(fbuf[f]); free(fmap[f]); free(flen[f]);
    }
    S->offs[si] = o;
    free(fbuf); free(fmap); free(flen);

    /* pairs */
    uint64_t nh = (uint64_t)(c->npairs * c->homolog_frac + 0.5);
    if (nh > c->npairs) nh = c->npairs;
    S->npairs = c->npairs;
    S->pairs = (pg_pair *)calloc(c->npairs ? c->npairs : 1, sizeof(pg_pair));
    S->homolog = (uint8_t *)calloc(c->npairs ? c->npairs : 1, 1);
    S->spurious = (uint8_t *)calloc(c->npairs ? c->npairs : 1, 1);
    /* homolog pairs: enumerate within-family pairs in a random family order, cycling */
    uint64_t ph = 0;
    if (nh > 0 && nfam > 0) {
        uint64_t *perm = (uint64_t *)malloc(nfam * sizeof(uint64_t));
        for (uint64_t f = 0; f < nfam; ++f) perm[f] = f;
        for (uint64_t f = nfam; f > 1; --f) {
            uint64_t g = ((uint64_t)rng_u32(&r0) * f) >> 32;
            uint64_t t = perm[f - 1]; perm[f - 1] = perm[g]; perm[g] = t;
        }
        int any = 0;
        for (uint64_t f = 0; f < nfam; ++f) if (fsz[f] >= 2) { any = 1; break; }
        uint64_t round = 0;
        while (any && ph < nh) {
            for (uint64_t q = 0; q < nfam && ph < nh; ++q) {
                uint64_t f = perm[q];
                uint32_t sz = fsz[f];
                if (sz < 2) continue;
                uint64_t npf = (uint64_t)sz * (sz - 1) / 2;
                if (round >= npf) continue;
                /* round-th pair (a < b) of this family */
                uint64_t idx = round, a = 0;
                while (idx >= (uint64_t)(sz - 1 - a)) { idx -= sz - 1 - a; ++a; }
                uint64_t b = a + 1 + idx;
                S->pairs[ph].row = (uint32_t)(fstart[f] + a);
                S->pairs[ph].col = (uint32_t)(fstart[f] + b);
                S->homolog[ph] = 1;
                ++ph;
            }
            ++round;
            if (round > (uint64_t)fam_max * fam_max) break;
        }
        free(perm);
    }
    for (uint64_t p = ph; p < c->npairs; ++p) {
        uint32_t a, b;
        int tries = 0;
        do {
            a = (uint32_t)(((uint64_t)rng_u32(&r0) * total) >> 32);
            b = (uint32_t)(((uint64_t)rng_u32(&r0) * total) >> 32);
        } while ((S->family[a] == S->family[b]) && nfam > 1 && ++tries < 100);
        S->pairs[p].row = a; S->pairs[p].col = b;
    }
    /* shuffle pair order so homologs and randoms interleave */
    for (uint64_t p = c->npairs; p > 1; --p) {
        uint64_t g = (uint64_t)(rng_unif(&r0) * (double)p);
        if (g >= p) g = p - 1;
        pg_pair t = S->pairs[p - 1]; S->pairs[p - 1] = S->pairs[g]; S->pairs[g] = t;
        uint8_t h = S->homolog[p - 1]; S->homolog[p - 1] = S->homolog[g]; S->homolog[g] = h;
    }
    /* seeds */
    if (c->k > 0) {
#pragma omp parallel
        {
            kmer_t *ka = (kmer_t *)malloc((c->len_max + 64) * sizeof(kmer_t));
            kmer_t *kb = (kmer_t *)malloc((c->len_max + 64) * sizeof(kmer_t));
            uint32_t *inv = (uint32_t *)calloc(65536, sizeof(uint32_t));
#pragma omp for schedule(dynamic, 256)
            for (long long p = 0; p < (long long)c->npairs; ++p) {
                pg_pair *pp = &S->pairs[p];
                rng_t r; rng_seed(&r, c->seed, 0x5eed0000000ULL + (uint64_t)p);
                const uint8_t *rs = S->seq + S->offs[pp->row];
                const uint8_t *cs = S->seq + S->offs[pp->col];
                uint32_t m = (uint32_t)(S->offs[pp->row + 1] - S->offs[pp->row]);
                uint32_t n = (uint32_t)(S->offs[pp->col + 1] - S->offs[pp->col]);
                const int hom = S->homolog[p] != 0;
                seed_pair(c, rs, m, cs, n, &r, ka, kb, pp, &S->spurious[p],
                          hom ? rootpos + S->offs[pp->row] : NULL,
                          hom ? rootpos + S->offs[pp->col] : NULL, inv);
            }
            free(ka); free(kb); free(inv);
        }
    }
    free(rootpos);
    free(fsz); free(fstart);
    return S;
}

uint64_t pg_synth_nseqs(const pg_synth *S) { return S->nseqs; }
uint64_t pg_synth_nres(const pg_synth *S) { return S->nres; }
uint64_t pg_synth_npairs(const pg_synth *S) { return S->npairs; }
const uint8_t *pg_synth_seq(const pg_synth *S) { return S->seq; }
const uint64_t *pg_synth_offs(const pg_synth *S) { return S->offs; }
const uint32_t *pg_synth_family(const pg_synth *S) { return S->family; }
const pg_pair *pg_synth_pairs(const pg_synth *S) { return S->pairs; }
const uint8_t *pg_synth_homolog(const pg_synth *S) { return S->homolog; }
const uint8_t *pg_synth_spurious(const pg_synth *S) { return S->spurious; }

void pg_synth_free(pg_synth *S)
{
    if (!S) return;
    free(S->seq); free(S->offs); free(S->family); free(S->pairs); free(S->homolog);
    free(S->spurious);
    free(S);
}
