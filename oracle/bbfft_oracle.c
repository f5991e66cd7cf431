/*
 * bbfft_oracle.c -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the reference's
 * double-batched FFT algorithm, used as the parity checker and as the timed CPU
 * baseline.  The product path never calls this code.
 *
 * What is restated (file:line in intel/double-batched-fft-library 0.5.1):
 *  - tensor layout and offsets m*s0 + n*s1 + k*s2      include/bbfft/configuration.hpp:151-192
 *  - trial-division factorisation                      src/base/prime_factorization.cpp:13-25
 *  - in-place mixed-radix stages (inplace<ESum>)        src/base/mixed_radix_fft.cpp:215-254
 *      for f = L-1..0: J /= Nf; for j, k: y[kf] = esum_kf * w_{J Nf}^{dir kf j}
 *  - pair-optimised e-sum (w and conj(w) share work)    src/base/mixed_radix_fft.cpp:55-126
 *  - unscrambling of the digit-reversed output          src/base/scrambler.hpp:67-101
 *  - real even N: N/2-point complex FFT + post-process  src/base/generator/sbfft_gen.cpp:162-200
 *                 pre-process + N/2-point FFT (c2r)     src/base/generator/sbfft_gen.cpp:202-247
 *  - real odd N: two K-slices packed into one FFT       src/base/generator/sbfft_gen.cpp:249-351
 *  - nd transforms as chained 1d passes                 src/common/algorithm/nd_fft.hpp:27-176
 *  - twiddles: exp(2 pi i e / n) computed in extended precision, rounded once
 *    (src/base/root_of_unity.cpp:144-189 and the exactly rounded LUT root_of_unity.hpp)
 *
 * Parity of this restatement is pinned by the reference's own known-answer tests
 * (test/c2c.cpp, test/r2c.cpp, test/callback.cpp) reimplemented in tests/, and by an
 * independent FP64 DFT.
 *
 * Build: make -C oracle  (liboracle.so)
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MAXF 64

typedef struct {
    int n;
    int nf;
    int f[MAXF];
} factorization;

/* reference src/base/prime_factorization.cpp:13-25 */
static void trial_division(int n, factorization *fz) {
    fz->n = n;
    fz->nf = 0;
    int f = 2;
    while (n > 1) {
        if (n % f == 0) {
            fz->f[fz->nf++] = f;
            n /= f;
        } else {
            ++f;
        }
    }
}

/* reference src/base/scrambler.hpp:67-101 (unscrambler, index in [0, N)) */
static int unscramble(const factorization *fz, int index) {
    if (fz->nf <= 1) {
        return index;
    }
    int result = 0;
    for (int i = fz->nf - 1; i >= 0; --i) {
        int Ni = fz->f[i];
        result = result * Ni + index % Ni;
        index /= Ni;
    }
    return result;
}

/* exp(2 pi i e / n) rounded once from long double */
static void root_of_unity(long e, long n, long double *c, long double *s) {
    long q = ((e % n) + n) % n;
    if ((4 * q) % n == 0) {
        static const int cs[4][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
        int quad = (int)((4 * q) / n);
        *c = cs[quad][0];
        *s = cs[quad][1];
        return;
    }
    const long double tau = 6.283185307179586476925286766559005768L;
    long double a = tau * (long double)q / (long double)n;
    *c = cosl(a);
    *s = sinl(a);
}

#define DEFINE_ORACLE(REAL, SFX)                                                                 \
    typedef struct {                                                                             \
        REAL re, im;                                                                             \
    } cx_##SFX;                                                                                  \
                                                                                                 \
    /* table of w_N^e = exp(2 pi i e / N), e = 0..N-1, rounded to REAL */                       \
    static cx_##SFX *make_table_##SFX(int N) {                                                   \
        cx_##SFX *t = (cx_##SFX *)malloc(sizeof(cx_##SFX) * (size_t)N);                          \
        for (int e = 0; e < N; ++e) {                                                            \
            long double c, s;                                                                    \
            root_of_unity(e, N, &c, &s);                                                         \
            t[e].re = (REAL)c;                                                                   \
            t[e].im = (REAL)s;                                                                   \
        }                                                                                        \
        return t;                                                                                \
    }                                                                                            \
                                                                                                 \
    /* w_{sub}^{e}, sub | N, from the N-table */                                                 \
    static inline cx_##SFX tw_##SFX(const cx_##SFX *t, int N, int sub, long e) {                 \
        long q = ((e % sub) + sub) % sub;                                                        \
        return t[q * (N / sub)];                                                                 \
    }                                                                                            \
                                                                                                 \
    /* reference src/base/mixed_radix_fft.cpp:215-254 with the pair e-sum (55-126); output  */ \
    /* left in digit-reversed order                                                         */ \
    static void mixed_radix_inplace_##SFX(cx_##SFX *x, const factorization *fz, int dir,         \
                                          const cx_##SFX *t, int Nt, cx_##SFX *y) {              \
        int N = fz->n;                                                                           \
        int J = N, K = 1;                                                                        \
        for (int f = fz->nf - 1; f >= 0; --f) {                                                  \
            int Nf = fz->f[f];                                                                   \
            J /= Nf;                                                                             \
            for (int j = 0; j < J; ++j) {                                                        \
                for (int k = 0; k < K; ++k) {                                                    \
                    /* indexer (J, Nf, K), column major: j + J jf + J Nf k */                    \
                    cx_##SFX *xb = x + j + (long)J * Nf * k;                                     \
                    for (int kf = 0; kf < Nf; ++kf) {                                            \
                        REAL sr = xb[0].re, si = xb[0].im;                                       \
                        if (kf == 0) {                                                           \
                            for (int jf = 1; jf < Nf; ++jf) {                                    \
                                sr += xb[(long)J * jf].re;                                       \
                                si += xb[(long)J * jf].im;                                       \
                            }                                                                    \
                        } else {                                                                 \
                            int h = (Nf - 1) / 2;                                                \
                            for (int jf = 1; jf <= h; ++jf) {                                    \
                                cx_##SFX w = tw_##SFX(t, Nt, Nf, (long)dir * kf * jf);            \
                                cx_##SFX a = xb[(long)J * jf], b = xb[(long)J * (Nf - jf)];      \
                                /* p11 = wr (a + b), p12 = wi * i * (a - b) */                   \
                                sr += w.re * (a.re + b.re) - w.im * (a.im - b.im);               \
                                si += w.re * (a.im + b.im) + w.im * (a.re - b.re);               \
                            }                                                                    \
                            if (Nf % 2 == 0) {                                                   \
                                cx_##SFX w = tw_##SFX(t, Nt, Nf, (long)dir * kf * (Nf / 2));      \
                                cx_##SFX a = xb[(long)J * (Nf / 2)];                             \
                                sr += a.re * w.re - a.im * w.im;                                 \
                                si += a.re * w.im + a.im * w.re;                                 \
                            }                                                                    \
                        }                                                                        \
                        cx_##SFX w = tw_##SFX(t, Nt, J * Nf, (long)dir * kf * j);                 \
                        y[kf].re = sr * w.re - si * w.im;                                        \
                        y[kf].im = sr * w.im + si * w.re;                                        \
                    }                                                                            \
                    for (int kf = 0; kf < Nf; ++kf) {                                            \
                        xb[(long)J * kf] = y[kf];                                                \
                    }                                                                            \
                }                                                                                \
            }                                                                                    \
            K *= Nf;                                                                             \
        }                                                                                        \
    }                                                                                            \
                                                                                                 \
    /* natural-order FFT of length N (unscrambled) */                                            \
    static void fft_##SFX(cx_##SFX *x, cx_##SFX *scratch, const factorization *fz, int dir,      \
                          const cx_##SFX *t, int Nt, cx_##SFX *y) {                              \
        mixed_radix_inplace_##SFX(x, fz, dir, t, Nt, y);                                         \
        for (int i = 0; i < fz->n; ++i) {                                                        \
            scratch[i] = x[unscramble(fz, i)];                                                   \
        }                                                                                        \
        memcpy(x, scratch, sizeof(cx_##SFX) * (size_t)fz->n);                                    \
    }                                                                                            \
                                                                                                 \
    typedef struct {                                                                             \
        int type, dir;                                                                           \
        long M, N, K;                                                                            \
        const void *in;                                                                          \
        void *out;                                                                               \
        long is1, is2, os1, os2;                                                                 \
        long k0, k1; /* range of K-slices (or K-slice pairs for odd real) */                    \
        const cx_##SFX *t;   /* table w_Nt */                                                    \
        const factorization *fz;                                                                 \
        int Nt;                                                                                  \
    } job_##SFX;                                                                                 \
                                                                                                 \
    static void run_job_##SFX(job_##SFX *jb) {                                                   \
        int N = (int)jb->N;                                                                      \
        int Nfft = jb->fz->n;                                                                    \
        cx_##SFX *x = (cx_##SFX *)malloc(sizeof(cx_##SFX) * (size_t)(Nfft + 1) * 3 + 64 * sizeof(cx_##SFX)); \
        cx_##SFX *scr = x + Nfft + 1;                                                            \
        cx_##SFX *y = scr + Nfft + 1;                                                            \
        const cx_##SFX *t = jb->t;                                                               \
        int Nt = jb->Nt;                                                                         \
        for (long kk = jb->k0; kk < jb->k1; ++kk) {                                              \
            for (long m = 0; m < jb->M; ++m) {                                                   \
                if (jb->type == 0) { /* c2c */                                                   \
                    const cx_##SFX *in = (const cx_##SFX *)jb->in + m + kk * jb->is2;            \
                    cx_##SFX *out = (cx_##SFX *)jb->out + m + kk * jb->os2;                      \
                    for (int n = 0; n < N; ++n) x[n] = in[n * jb->is1];                          \
                    fft_##SFX(x, scr, jb->fz, jb->dir, t, Nt, y);                                    \
                    for (int n = 0; n < N; ++n) out[n * jb->os1] = x[n];                         \
                } else if (jb->type == 1 && N % 2 == 0) { /* r2c half, sbfft_gen.cpp:162-200 */ \
                    const REAL *in = (const REAL *)jb->in + m + kk * jb->is2;                    \
                    cx_##SFX *out = (cx_##SFX *)jb->out + m + kk * jb->os2;                      \
                    int Nh = N / 2;                                                              \
                    for (int n = 0; n < Nh; ++n) {                                               \
                        x[n].re = in[(2 * n) * jb->is1];                                         \
                        x[n].im = in[(2 * n + 1) * jb->is1];                                     \
                    }                                                                            \
                    fft_##SFX(x, scr, jb->fz, -1, t, Nt, y);                                         \
                    for (int i = 0; i <= N / 4; ++i) {                                           \
                        int io = Nh - i;                                                         \
                        cx_##SFX y1 = x[i % Nh], y2 = x[io % Nh];                                \
                        y2.im = -y2.im;                                                          \
                        cx_##SFX a = {(y2.re + y1.re) / (REAL)2, (y2.im + y1.im) / (REAL)2};     \
                        cx_##SFX b = {(y2.re - y1.re) / (REAL)2, (y2.im - y1.im) / (REAL)2};     \
                        /* tw = power_of_w(-i, N) * i */                                         \
                        cx_##SFX w = tw_##SFX(t, Nt, N, -i);                                     \
                        cx_##SFX iw = {-w.im, w.re};                                             \
                        cx_##SFX bb = {b.re * iw.re - b.im * iw.im, b.re * iw.im + b.im * iw.re}; \
                        out[i * jb->os1].re = a.re + bb.re;                                      \
                        out[i * jb->os1].im = a.im + bb.im;                                      \
                        if (i != io) {                                                           \
                            out[io * jb->os1].re = a.re - bb.re;                                 \
                            out[io * jb->os1].im = bb.im - a.im;                                 \
                        }                                                                        \
                    }                                                                            \
                } else if (jb->type == 2 && N % 2 == 0) { /* c2r half, sbfft_gen.cpp:202-247 */ \
                    const cx_##SFX *in = (const cx_##SFX *)jb->in + m + kk * jb->is2;            \
                    REAL *out = (REAL *)jb->out + m + kk * jb->os2;                              \
                    int Nh = N / 2;                                                              \
                    for (int i = 0; i <= N / 4; ++i) {                                           \
                        int io = Nh - i;                                                         \
                        cx_##SFX x1 = in[i * jb->is1];                                           \
                        if (i == 0) x1.im = 0;                                                   \
                        cx_##SFX x2 = in[io * jb->is1];                                          \
                        x2.im = -x2.im;                                                          \
                        cx_##SFX a = {x1.re + x2.re, x1.im + x2.im};                             \
                        cx_##SFX b = {x1.re - x2.re, x1.im - x2.im};                             \
                        cx_##SFX w = tw_##SFX(t, Nt, N, i); /* power_of_w(i, N) * i */           \
                        cx_##SFX iw = {-w.im, w.re};                                             \
                        cx_##SFX bb = {b.re * iw.re - b.im * iw.im, b.re * iw.im + b.im * iw.re}; \
                        int is = i % Nh, ios = io % Nh;                                          \
                        x[is].re = a.re + bb.re;                                                 \
                        x[is].im = a.im + bb.im;                                                 \
                        if (is != ios) {                                                         \
                            x[ios].re = a.re - bb.re;                                            \
                            x[ios].im = bb.im - a.im;                                            \
                        }                                                                        \
                    }                                                                            \
                    fft_##SFX(x, scr, jb->fz, 1, t, Nt, y);                                          \
                    for (int n = 0; n < Nh; ++n) {                                               \
                        out[(2 * n) * jb->os1] = x[n].re;                                        \
                        out[(2 * n + 1) * jb->os1] = x[n].im;                                    \
                    }                                                                            \
                } else if (jb->type == 1) { /* r2c odd: slices 2kk, 2kk+1, sbfft_gen.cpp:249-291 */ \
                    long ka = 2 * kk, kb = 2 * kk + 1;                                           \
                    const REAL *ina = (const REAL *)jb->in + m + ka * jb->is2;                   \
                    const REAL *inb = (const REAL *)jb->in + m + kb * jb->is2;                   \
                    for (int n = 0; n < N; ++n) {                                                \
                        x[n].re = ina[n * jb->is1];                                              \
                        x[n].im = kb < jb->K ? inb[n * jb->is1] : (REAL)0;                       \
                    }                                                                            \
                    fft_##SFX(x, scr, jb->fz, -1, t, Nt, y);                                         \
                    cx_##SFX *outa = (cx_##SFX *)jb->out + m + ka * jb->os2;                     \
                    cx_##SFX *outb = (cx_##SFX *)jb->out + m + kb * jb->os2;                     \
                    for (int i = 0; i <= N / 2; ++i) {                                           \
                        int io = (N - i) % N;                                                    \
                        cx_##SFX y1 = x[i], y2 = x[io];                                          \
                        y2.im = -y2.im;                                                          \
                        cx_##SFX a = {(y2.re + y1.re) / (REAL)2, (y2.im + y1.im) / (REAL)2};     \
                        cx_##SFX b = {(y2.re - y1.re) / (REAL)2, (y2.im - y1.im) / (REAL)2};     \
                        outa[i * jb->os1] = a;                                                   \
                        if (kb < jb->K) {                                                        \
                            outb[i * jb->os1].re = -b.im;                                        \
                            outb[i * jb->os1].im = b.re;                                         \
                        }                                                                        \
                    }                                                                            \
                } else { /* c2r odd: sbfft_gen.cpp:293-351 */                                    \
                    long ka = 2 * kk, kb = 2 * kk + 1;                                           \
                    const cx_##SFX *ina = (const cx_##SFX *)jb->in + m + ka * jb->is2;           \
                    const cx_##SFX *inb = (const cx_##SFX *)jb->in + m + kb * jb->is2;           \
                    for (int i = 0; i <= N / 2; ++i) {                                           \
                        int io = (N - i) % N;                                                    \
                        cx_##SFX xa = ina[i * jb->is1];                                          \
                        cx_##SFX xb = kb < jb->K ? inb[i * jb->is1] : (cx_##SFX){0, 0};          \
                        if (i == 0) {                                                            \
                            xa.im = 0;                                                           \
                            xb.im = 0;                                                           \
                        }                                                                        \
                        cx_##SFX ib = {-xb.im, xb.re}; /* i * xb */                              \
                        x[i].re = xa.re + ib.re;                                                 \
                        x[i].im = xa.im + ib.im;                                                 \
                        if (i != io) {                                                           \
                            x[io].re = xa.re - ib.re;                                            \
                            x[io].im = -(xa.im - ib.im);                                         \
                        }                                                                        \
                    }                                                                            \
                    fft_##SFX(x, scr, jb->fz, 1, t, Nt, y);                                          \
                    REAL *outa = (REAL *)jb->out + m + ka * jb->os2;                             \
                    REAL *outb = (REAL *)jb->out + m + kb * jb->os2;                             \
                    for (int n = 0; n < N; ++n) {                                                \
                        outa[n * jb->os1] = x[n].re;                                             \
                        if (kb < jb->K) outb[n * jb->os1] = x[n].im;                             \
                    }                                                                            \
                }                                                                                \
            }                                                                                    \
        }                                                                                        \
        free(x);                                                                                 \
    }                                                                                            \
                                                                                                 \
    static void *thread_main_##SFX(void *arg) {                                                  \
        run_job_##SFX((job_##SFX *)arg);                                                         \
        return NULL;                                                                             \
    }                                                                                            \
                                                                                                 \
    /* One double-batched 1d pass.  type: 0 c2c, 1 r2c, 2 c2r.  Strides in elements.       */   \
    int oracle_fft1d_##SFX(int type, int dir, long M, long N, long K, const void *in, long is1,  \
                           long is2, void *out, long os1, long os2, int threads) {               \
        if (N < 1 || M < 1 || K < 1 || type < 0 || type > 2) return -1;                         \
        int real = type != 0;                                                                    \
        int Nfft = (real && N % 2 == 0) ? (int)(N / 2) : (int)N;                                 \
        int Nt = real && N % 2 == 0 ? (int)N : Nfft;                                             \
        factorization fz;                                                                        \
        trial_division(Nfft, &fz);                                                               \
        cx_##SFX *t = make_table_##SFX(Nt);                                                      \
        long Kw = (real && N % 2 == 1) ? (K + 1) / 2 : K;                                        \
        if (threads < 1) threads = 1;                                                            \
        if (threads > Kw) threads = (int)Kw;                                                     \
        job_##SFX *jobs = (job_##SFX *)calloc((size_t)threads, sizeof(job_##SFX));               \
        pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));                \
        for (int i = 0; i < threads; ++i) {                                                      \
            job_##SFX *jb = &jobs[i];                                                            \
            jb->type = type;                                                                     \
            jb->dir = dir;                                                                       \
            jb->M = M;                                                                           \
            jb->N = N;                                                                           \
            jb->K = K;                                                                           \
            jb->in = in;                                                                         \
            jb->out = out;                                                                       \
            jb->is1 = is1;                                                                       \
            jb->is2 = is2;                                                                       \
            jb->os1 = os1;                                                                       \
            jb->os2 = os2;                                                                       \
            jb->k0 = Kw * i / threads;                                                           \
            jb->k1 = Kw * (i + 1) / threads;                                                     \
            jb->t = t;                                                                           \
            jb->fz = &fz;                                                                        \
            jb->Nt = Nt;                                                                         \
        }                                                                                        \
        if (threads == 1) {                                                                      \
            run_job_##SFX(&jobs[0]);                                                             \
        } else {                                                                                 \
            for (int i = 0; i < threads; ++i)                                                    \
                pthread_create(&tid[i], NULL, thread_main_##SFX, &jobs[i]);                      \
            for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);                        \
        }                                                                                        \
        free(tid);                                                                               \
        free(jobs);                                                                              \
        free(t);                                                                                 \
        return 0;                                                                                \
    }

DEFINE_ORACLE(double, f64)
DEFINE_ORACLE(float, f32)
