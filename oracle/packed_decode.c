/*
 * Standardised decode of PLINK SNP rows for the FP64 oracle -- TEST
 * INFRASTRUCTURE ONLY (never linked into the product library).
 *
 * decode_single_snp (src/bed.rs:300-379) with mean imputation: sample s of a
 * SNP row sits in byte s/4 at bit offset 2*(s%4) (src/bed.rs:262-281); code
 * 00 -> 0, 01 -> missing, 10 -> 1, 11 -> 2 (DECODE_TABLE, src/bed.rs:16); an
 * observed call becomes (g - mean) * scale and a missing call 0.  The
 * per-SNP mean and scale are inputs (the oracle derives them from integer
 * allele counts).  Rows are split over host threads; each value is computed
 * by the same two FP64 operations as the NumPy restatement.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct {
    const uint8_t* packed;
    uint64_t bps;
    const int64_t* rows;
    uint64_t r0, r1, n;
    const double* mean;
    const double* scale;
    double* out;
} job_t;

static void* run(void* arg) {
    const job_t* j = (const job_t*)arg;
    for (uint64_t r = j->r0; r < j->r1; ++r) {
        const uint8_t* src = j->packed + (uint64_t)j->rows[r] * j->bps;
        const double m = j->mean[r], s = j->scale[r];
        const double v[4] = {(0.0 - m) * s, 0.0, (1.0 - m) * s, (2.0 - m) * s};
        double* dst = j->out + r * j->n;
        for (uint64_t i = 0; i < j->n; ++i) dst[i] = v[(src[i >> 2] >> (2 * (i & 3))) & 3];
    }
    return NULL;
}

/* out (c x n, row-major) = standardised rows rows[0..c) of packed (bps bytes
 * per row); returns 0, or -1 if a thread could not be started. */
int oracle_decode_rows(const uint8_t* packed, uint64_t bps, const int64_t* rows, uint64_t c, uint64_t n,
                       const double* mean, const double* scale, double* out, int threads) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > c) threads = c ? (int)c : 1;
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    job_t* jobs = (job_t*)malloc(sizeof(job_t) * (size_t)threads);
    if (!tid || !jobs) {
        free(tid);
        free(jobs);
        return -1;
    }
    int started = 0, rc = 0;
    for (int t = 0; t < threads; ++t) {
        /* jobs run on threads tid[0..started) or inline */
        job_t* j = &jobs[t];
        j->packed = packed;
        j->bps = bps;
        j->rows = rows;
        j->r0 = c * (uint64_t)t / (uint64_t)threads;
        j->r1 = c * (uint64_t)(t + 1) / (uint64_t)threads;
        j->n = n;
        j->mean = mean;
        j->scale = scale;
        j->out = out;
        if (t + 1 == threads) {
            run(j);
        } else if (pthread_create(&tid[started], NULL, run, j) == 0) {
            ++started;
        } else {
            run(j);
        }
    }
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
    return rc;
}
