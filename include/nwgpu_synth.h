/*
 * nwgpu_synth.h -- seeded synthetic protein families (host-only helper).
 *
 * Not part of the reference's interface: the reference reads real FASTA files
 * (FastaFile.cpp) and ships no generator.  This library generates the seeded
 * workloads the benchmarks and tests run on; see synth.cpp for the model.
 */
#ifndef NWGPU_SYNTH_H
#define NWGPU_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { NWS_ROOT_FIXED = 0, NWS_ROOT_UNIFORM = 1, NWS_ROOT_LOGNORMAL = 2 };

typedef struct {
  int32_t families;     /* independent families                              */
  int32_t per_family;   /* leaves per family (sequences)                      */
  int32_t root_mode;    /* NWS_ROOT_*                                         */
  int32_t clip_lo;      /* length clip                                        */
  int32_t clip_hi;
  int32_t pad;
  double root_a;        /* fixed length | uniform low | lognormal median      */
  double root_b;        /* -            | uniform high| lognormal sigma       */
  double ps;            /* per-edge, per-site substitution probability        */
  double pi;            /* per-edge, per-site indel probability               */
} nws_spec;

typedef struct {
  int32_t n;            /* sequences                                          */
  int32_t pad;
  int64_t total;        /* residues                                           */
  char* residues;       /* concatenated ASCII residues (no separators)        */
  int32_t* lengths;     /* n lengths                                          */
} nws_out;

/* Generate; 0 on success.  Release with nws_release. */
int nws_generate(const nws_spec* spec, uint64_t seed, nws_out* out);
void nws_release(nws_out* out);

/* Shapes of the benchmark configurations 0..3 and their seeds. */
int nws_config_spec(int cfg, nws_spec* spec);
uint64_t nws_config_seed(int cfg);

#ifdef __cplusplus
}
#endif
#endif
