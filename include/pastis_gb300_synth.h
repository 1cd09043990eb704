/*
 * pastis_gb300_synth.h -- seeded synthetic protein families and candidate pairs
 * (stand-in for the reference's FASTA input and k-mer SpGEMM output).
 */
#ifndef PASTIS_GB300_SYNTH_H
#define PASTIS_GB300_SYNTH_H

#include <stdint.h>
#include "pastis_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pg_synth_cfg {
    uint64_t seed;
    uint64_t nseqs;            /* proteins generated (grouped in families) */
    uint32_t fam_min, fam_max; /* family size range (a root and mutated members) */
    double   len_median, len_sigma;  /* lognormal root lengths */
    uint32_t len_min, len_max;       /* clamp */
    double   mix_frac;         /* fraction of roots with uniform lengths instead */
    uint32_t mix_lo, mix_hi;
    double   id_lo, id_hi;     /* member identity to the root, uniform */
    double   indel_rate;       /* indel events per residue */
    double   indel_mean;       /* geometric indel length mean */
    uint64_t npairs;
    double   homolog_frac;     /* share of within-family pairs */
    uint32_t k;                /* seed k-mer length (0: no seeds) */
    int32_t  alph;             /* seeding alphabet: 0 = full, 1 = murphy10 */
} pg_synth_cfg;

typedef struct pg_synth pg_synth;

pg_synth *pg_synth_generate(const pg_synth_cfg *cfg);
void      pg_synth_free(pg_synth *s);
uint64_t  pg_synth_nseqs(const pg_synth *s);
uint64_t  pg_synth_nres(const pg_synth *s);
uint64_t  pg_synth_npairs(const pg_synth *s);
const uint8_t  *pg_synth_seq(const pg_synth *s);      /* residue codes 0..19 */
const uint64_t *pg_synth_offs(const pg_synth *s);     /* nseqs + 1 */
const uint32_t *pg_synth_family(const pg_synth *s);
const pg_pair  *pg_synth_pairs(const pg_synth *s);
const uint8_t  *pg_synth_homolog(const pg_synth *s);  /* 1 = within-family pair */
const uint8_t  *pg_synth_spurious(const pg_synth *s); /* 1 = no shared k-mer, random seed */

#ifdef __cplusplus
}
#endif
#endif
