/*
 * oracle/direct.c -- CPU oracle of the masked distance map in Float64, direct summation.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by oracle/iqsim_oracle.py for the tests, smoke() and the
 * CPU baseline of bench.py. It is never linked into the product library.
 *
 * fastdistance (src/utils.jl:5-13) is |sum_k w_k img[p+k]^2 - 2 sum_k w_k kern_k img[p+k] +
 * sum_k w_k kern_k^2|, which for 0/1 weights equals sum over the mask of (img[p+k] - kern_k)^2.
 * The reference evaluates it with FFT correlations (src/imfilter.jl:5-26), whose Float64
 * rounding depends on the FFT library; this oracle fixes one exact evaluation instead:
 *
 *   D[p] = 0;  for each offset k of the mask, in column-major order (x fastest):
 *                d = img[p + k] - kern[k];  D[p] = D[p] + (w_k == 1 ? d * d : (w_k * d) * d)
 *
 * every operation a separately rounded IEEE Float64 operation (compiled with
 * -ffp-contract=off, no fused multiply-add). The library's exact re-rank evaluates the same
 * sequence, so both give the same bits; it differs from the exact real value by at most
 * (K + 2) * 2^-53 relative (no cancellation: every term is non-negative).
 *
 * Arrays are column-major with extents (nx, ny, nz); the output has the valid extents
 * (nx - tx + 1, ny - ty + 1, nz - tz + 1). Output planes are split over `nthreads` threads.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct {
    const double *img;
    long long nx, ny, nz;
    const double *kv;      /* values of the mask offsets, in order */
    const double *kw;      /* weights of the mask offsets */
    const long long *koff; /* linear image offsets of the mask offsets */
    long long K;
    long long ox, oy, oz;  /* output extents */
    double *out;
    long long z0, z1;      /* output planes of this thread */
} job_t;

static void *run(void *arg) {
    const job_t *j = (const job_t *)arg;
    const long long sx = j->nx, sxy = j->nx * j->ny;
    for (long long z = j->z0; z < j->z1; z++)
        for (long long y = 0; y < j->oy; y++) {
            double *o = j->out + j->ox * (y + j->oy * z);
            const double *base = j->img + sx * y + sxy * z;
            for (long long x = 0; x < j->ox; x++) o[x] = 0.0;
            for (long long k = 0; k < j->K; k++) {
                const double v = j->kv[k], w = j->kw[k];
                const double *src = base + j->koff[k];
                if (w == 1.0) {
                    for (long long x = 0; x < j->ox; x++) {
                        const double d = src[x] - v;
                        o[x] = o[x] + d * d;
                    }
                } else {
                    for (long long x = 0; x < j->ox; x++) {
                        const double d = src[x] - v;
                        o[x] = o[x] + (w * d) * d;
                    }
                }
            }
        }
    return NULL;
}

/*
 * img: nx*ny*nz doubles; kern, wts: tx*ty*tz doubles (weights 0 skip the offset);
 * out: ox*oy*oz doubles. Returns 0, or -1 on bad sizes / allocation failure.
 */
int oracle_direct_ssd(const double *img, long long nx, long long ny, long long nz,
                      const double *kern, const double *wts, long long tx, long long ty,
                      long long tz, double *out, int nthreads) {
    if (tx < 1 || ty < 1 || tz < 1 || tx > nx || ty > ny || tz > nz) return -1;
    const long long ox = nx - tx + 1, oy = ny - ty + 1, oz = nz - tz + 1;
    const long long T = tx * ty * tz;
    double *kv = (double *)malloc(sizeof(double) * (size_t)T);
    double *kw = (double *)malloc(sizeof(double) * (size_t)T);
    long long *koff = (long long *)malloc(sizeof(long long) * (size_t)T);
    if (!kv || !kw || !koff) {
        free(kv); free(kw); free(koff);
        return -1;
    }
    long long K = 0;
    for (long long z = 0; z < tz; z++)
        for (long long y = 0; y < ty; y++)
            for (long long x = 0; x < tx; x++) {
                const long long t = x + tx * (y + ty * z);
                if (wts[t] == 0.0) continue;
                kv[K] = kern[t];
                kw[K] = wts[t];
                koff[K] = x + nx * (y + ny * z);
                K++;
            }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > oz) nthreads = (int)oz;
    if (nthreads > 64) nthreads = 64;
    job_t jobs[64];
    pthread_t th[64];
    for (int i = 0; i < nthreads; i++) {
        job_t *j = &jobs[i];
        j->img = img; j->nx = nx; j->ny = ny; j->nz = nz;
        j->kv = kv; j->kw = kw; j->koff = koff; j->K = K;
        j->ox = ox; j->oy = oy; j->oz = oz; j->out = out;
        j->z0 = oz * i / nthreads;
        j->z1 = oz * (i + 1) / nthreads;
    }
    int started = 0;
    for (int i = 1; i < nthreads; i++) {
        if (pthread_create(&th[i], NULL, run, &jobs[i]) != 0) break;
        started = i;
    }
    /* planes of threads that failed to start run here, after this thread's own */
    run(&jobs[0]);
    for (int i = started + 1; i < nthreads; i++) run(&jobs[i]);
    for (int i = 1; i <= started; i++) pthread_join(th[i], NULL);
    free(kv); free(kw); free(koff);
    return 0;
}
