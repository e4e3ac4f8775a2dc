/*
 * swgsynth — seeded synthetic genomes and reads for tests and benchmarks.
 *
 * The reference ships no data (its README's read generator is absent), so
 * every workload here is generated: a random genome (GC content, optional
 * repeat families and tandem repeats), reads of fixed length sampled
 * uniformly from both strands with iid substitutions and single-base indels,
 * written as single-line FASTA: ">r<i>\n<bases>\n" per read.
 * Output depends only on the parameters (not on the thread count).
 */
#ifndef SWG_SYNTH_H
#define SWG_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct swg_synth_params {
    uint64_t seed;
    uint64_t genome_len;
    double gc;                  /* G+C fraction of the background genome */
    double repeat_frac;         /* fraction of the genome written by repeat families */
    uint32_t repeat_unit_min;   /* family unit length, log-uniform in [min,max] */
    uint32_t repeat_unit_max;
    uint32_t repeat_copies_min; /* copies per family, uniform in [min,max] */
    uint32_t repeat_copies_max;
    double repeat_divergence;   /* per-base mutation rate of each copy */
    double tandem_frac;         /* fraction of the genome in tandem arrays */
    uint32_t tandem_unit_min;   /* tandem unit length, uniform in [min,max] */
    uint32_t tandem_unit_max;
    uint32_t tandem_len_min;    /* array length, log-uniform in [min,max] */
    uint32_t tandem_len_max;
    uint64_t n_reads;
    uint32_t read_len;
    double sub_rate;   /* per-base substitution probability */
    double indel_rate; /* per-base single-base indel probability (half ins, half del) */
    int threads;       /* 0 = all cores */
} swg_synth_params;

/* Fill p with the defaults: uniform genome (gc 0.5), no repeats, no errors. */
void swg_synth_defaults(swg_synth_params *p);
/* Generate FASTA into a malloc'd buffer; returns its length or -1. */
int64_t swg_synth_fasta(const swg_synth_params *p, char **out);
/* Generate and write to a file; returns bytes written or -1. */
int64_t swg_synth_fasta_file(const swg_synth_params *p, const char *path);
void swg_synth_free(char *buf);

#ifdef __cplusplus
}
#endif
#endif
