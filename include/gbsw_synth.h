/*
 * gbsw_synth.h -- seeded synthetic alignment workloads.
 *
 * Not part of the reference's interface: the reference ships no generator
 * (its DNA test inputs and protein references are absent).  These pairs stand
 * in for them in the tests and the benchmark.  Host-only code, built into
 * libgbsw_synth.so.
 */
#ifndef GBSW_SYNTH_H
#define GBSW_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSW_SYNTH_DNA 0
#define GBSW_SYNTH_PROTEIN 1

#define GBSW_SYNTH_UNIFORM 0
#define GBSW_SYNTH_LOGNORMAL 1

#define GBSW_SYNTH_MAX_COMPONENTS 4

typedef struct {
    int32_t dist;   /* GBSW_SYNTH_UNIFORM on [min,max] or GBSW_SYNTH_LOGNORMAL   */
    int32_t min;    /* clip bounds (inclusive)                                  */
    int32_t max;
    double median;  /* log-normal only                                          */
    double sigma;
} gbsw_synth_len;

typedef struct {
    double weight;              /* mixture weight                                  */
    int32_t alphabet;           /* GBSW_SYNTH_DNA / GBSW_SYNTH_PROTEIN             */
    int32_t query_from_ref_length; /* related queries copy the whole reference      */
    gbsw_synth_len ref_len;
    gbsw_synth_len query_len;
    double related_fraction;    /* share of queries mutated from their reference   */
    double substitution_rate;   /* per position (DNA; protein when identity <= 0)  */
    double target_identity;     /* protein: solve the substitution rate for this   */
    double indel_rate;          /* indel events per position                       */
    double indel_mean;          /* mean indel length (geometric on 1, 2, ...)      */
} gbsw_synth_component;

typedef struct {
    int32_t ncomponents;
    gbsw_synth_component components[GBSW_SYNTH_MAX_COMPONENTS];
    double aa_background[20];   /* residue frequencies, order ARNDCQEGHILKMFPSTWYV */
    int32_t aa_matrix[400];     /* 20x20 substitution scores in the same order     */
} gbsw_synth_params;

typedef struct {
    int64_t n;
    char* ref;           /* concatenated references                         */
    int64_t* ref_off;    /* n+1 exclusive prefix offsets                    */
    char* query;         /* concatenated queries                            */
    int64_t* query_off;  /* n+1 exclusive prefix offsets                    */
    int32_t* component;  /* mixture component of each pair                  */
    int64_t ref_total;
    int64_t query_total;
} gbsw_synth_batch;

/* Returns 0, -1 on bad parameters, -2 on allocation failure.  Free with
 * gbsw_synth_free. */
int gbsw_synth_generate(const gbsw_synth_params* params, int64_t n, uint64_t seed,
                        gbsw_synth_batch* out);
void gbsw_synth_free(gbsw_synth_batch* batch);

#ifdef __cplusplus
}
#endif
#endif
