/*
 * oracle_fft.c - CPU oracle for the aclfft transform path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; it is used by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's CPU-baseline leg.  The GPU product path fails
 * loudly when its CUDA library is missing instead of falling back here.
 *
 * Two families of functions:
 *
 *  orc_*   FP64 checker.  A mixed-radix decimation-in-time FFT (smallest prime
 *          factor first, direct O(p^2) sub-DFT for each prime p) with twiddles
 *          computed in double from an exactly reduced integer angle.  The
 *          real-input and real-output transforms restate the reference's own
 *          algorithms:
 *            R2C, even n: pack x[2k] + i x[2k+1], n/2-point C2C, then the
 *              even/odd post-process with X[0] = Re Z0 + Im Z0,
 *              X[n/2] = Re Z0 - Im Z0 and zero imaginary parts at both ends
 *              (src/rfft1_d/arch35/fft/rfft1_d_fft_kernel.h:39-65,169-228);
 *            R2C, odd n: full complex FFT of (x, 0), keep bins 0..n/2
 *              (same file :67-87, :230-252);
 *            C2R: Hermitian expansion to n bins, full inverse C2C, real part,
 *              no 1/n scaling
 *              (src/irfft1_d/arch35/fft/irfft1_d_fft_kernel.h:40-77,162-178);
 *            2D: forward/backward C2C over both axes of a row-major
 *              [batch][nx][ny] array (the golden of
 *              src/fft2_d/tests/fft2_d_data/gen_data.py:47-68);
 *            VERTICAL 1D: transforms down the columns of [n][batch]
 *              (src/fft1_d/tests/fft1_d_data/gen_data.py:79-84).
 *
 *  port_*  FP32 port of the reference's arch35 mixed-radix Stockham path,
 *          used only as the timed CPU baseline.  Stages are chosen greedily
 *          by smallest prime (src/fft1_d/arch35/fft/fft1_d_c2c.cpp:23-42),
 *          each stage is an autosort Stockham pass
 *          y[block*len + q*prev + j] = sum_p D(q,p) tw(p,j) x[block*prev + j + p*part]
 *          (src/fft1_d/arch35/mix/fft1_d_c2c_mix_kernel.h:29-120,1051-1186)
 *          with the DFT and twiddle tables generated in double and rounded
 *          to float (src/fft1_d/arch35/mix/fft1_d_c2c_mix.cpp:74-125).
 *
 * Complex data is interleaved (re, im).  All functions return 0 on success
 * and a negative value on bad arguments or allocation failure.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double re, im;
} cd;

/* exp(sign * 2*pi*i * num/den) with the angle reduced exactly in integers and
 * folded into the first octant before calling sin/cos. */
static cd unit_root(int64_t num, int64_t den, int sign)
{
    int64_t m = num % den;
    if (m < 0) m += den;
    /* angle = 2*pi*m/den; work in units of 1/(8*den) of a full turn */
    int64_t e = 8 * m; /* position in eighths-of-turn * den */
    int oct = (int)(e / den);
    int64_t rem = e - (int64_t)oct * den; /* [0, den) within the octant */
    double frac = (double)rem / (double)den; /* [0,1) of an octant */
    double a = frac * (M_PI / 4.0);
    double c, s;
    /* angle = oct*pi/4 + a */
    double ca = cos(a), sa = sin(a);
    double cb = cos(M_PI / 4.0 - a), sb = sin(M_PI / 4.0 - a);
    switch (oct & 7) {
    case 0: c = ca; s = sa; break;
    case 1: c = sb; s = cb; break;
    case 2: c = -sa; s = ca; break;
    case 3: c = -cb; s = sb; break;
    case 4: c = -ca; s = -sa; break;
    case 5: c = -sb; s = -cb; break;
    case 6: c = sa; s = -ca; break;
    default: c = cb; s = -sb; break;
    }
    cd r = {c, sign < 0 ? -s : s};
    return r;
}

static int64_t smallest_prime_factor(int64_t n)
{
    if (n % 2 == 0) return 2;
    for (int64_t f = 3; f * f <= n; f += 2)
        if (n % f == 0) return f;
    return n;
}

/* y[0..n) = DFT_n of x[0], x[xs], ...; tw[j] = W_N^j with N = n * tstep. */
static void fft_rec(const cd* x, int64_t xs, cd* y, int64_t n, const cd* tw, int64_t tstep, int64_t N, cd* tmp)
{
    if (n == 1) {
        y[0] = x[0];
        return;
    }
    int64_t p = smallest_prime_factor(n);
    int64_t m = n / p;
    if (m == 1) {
        /* direct prime DFT */
        for (int64_t k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (int64_t j = 0; j < n; ++j) {
                int64_t idx = ((j * k) % n) * tstep;
                cd w = tw[idx % N];
                cd v = x[j * xs];
                sr += v.re * w.re - v.im * w.im;
                si += v.re * w.im + v.im * w.re;
            }
            tmp[k].re = sr;
            tmp[k].im = si;
        }
        memcpy(y, tmp, (size_t)n * sizeof(cd));
        return;
    }
    for (int64_t r = 0; r < p; ++r) fft_rec(x + r * xs, xs * p, y + r * m, m, tw, tstep * p, N, tmp);
    /* X[k + m*q] = sum_r W_n^{r*(k + m*q)} Y_r[k] */
    cd* t = tmp;           /* p entries */
    cd* out = tmp + p;     /* n entries */
    for (int64_t k = 0; k < m; ++k) {
        for (int64_t r = 0; r < p; ++r) {
            cd w = tw[((r * k) % n) * tstep % N];
            cd v = y[r * m + k];
            t[r].re = v.re * w.re - v.im * w.im;
            t[r].im = v.re * w.im + v.im * w.re;
        }
        for (int64_t q = 0; q < p; ++q) {
            double sr = 0.0, si = 0.0;
            for (int64_t r = 0; r < p; ++r) {
                cd w = tw[((r * q) % p) * m * tstep % N];
                sr += t[r].re * w.re - t[r].im * w.im;
                si += t[r].re * w.im + t[r].im * w.re;
            }
            out[k + m * q].re = sr;
            out[k + m * q].im = si;
        }
    }
    memcpy(y, out, (size_t)n * sizeof(cd));
}

static cd* make_table(int64_t n, int sign)
{
    cd* tw = (cd*)malloc((size_t)n * sizeof(cd));
    if (!tw) return NULL;
    for (int64_t j = 0; j < n; ++j) tw[j] = unit_root(j, n, sign);
    return tw;
}

/* One transform of length n, input at stride xs (in cd units), output
 * contiguous. */
static int c2c_one(const cd* x, int64_t xs, cd* y, int64_t n, const cd* tw)
{
    int64_t p = smallest_prime_factor(n);
    cd* tmp = (cd*)malloc((size_t)(n + (p > n ? p : n) + 8) * sizeof(cd));
    if (!tmp) return -2;
    fft_rec(x, xs, y, n, tw, 1, n, tmp);
    free(tmp);
    return 0;
}

/* Batched contiguous C2C: in/out are [batch][n] interleaved doubles.
 * sign = -1 forward, +1 backward (unscaled). */
int orc_c2c(const double* in, double* out, int64_t n, int64_t batch, int sign)
{
    if (n <= 0 || batch <= 0 || !in || !out) return -1;
    cd* tw = make_table(n, sign);
    if (!tw) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (int64_t b = 0; b < batch; ++b) {
        const cd* x = (const cd*)in + b * n;
        cd* y = (cd*)out + b * n;
        if (x == y) {
            cd* tmpx = (cd*)malloc((size_t)n * sizeof(cd));
            if (!tmpx) { err |= 1; continue; }
            memcpy(tmpx, x, (size_t)n * sizeof(cd));
            err |= c2c_one(tmpx, 1, y, n, tw) ? 1 : 0;
            free(tmpx);
        } else {
            err |= c2c_one(x, 1, y, n, tw) ? 1 : 0;
        }
    }
    free(tw);
    return err ? -2 : 0;
}

/* VERTICAL layout: in/out are [n][batch]; transform b is column b. */
int orc_c2c_vertical(const double* in, double* out, int64_t n, int64_t batch, int sign)
{
    if (n <= 0 || batch <= 0 || !in || !out) return -1;
    cd* tw = make_table(n, sign);
    if (!tw) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (int64_t b = 0; b < batch; ++b) {
        cd* col = (cd*)malloc((size_t)n * sizeof(cd));
        if (!col) { err |= 1; continue; }
        err |= c2c_one((const cd*)in + b, batch, col, n, tw) ? 1 : 0;
        for (int64_t i = 0; i < n; ++i) ((cd*)out)[i * batch + b] = col[i];
        free(col);
    }
    free(tw);
    return err ? -2 : 0;
}

/* 2D C2C over [batch][nx][ny]: rows (length ny) then columns (length nx). */
int orc_c2c_2d(const double* in, double* out, int64_t nx, int64_t ny, int64_t batch, int sign)
{
    if (nx <= 0 || ny <= 0 || batch <= 0 || !in || !out) return -1;
    int rc = orc_c2c(in, out, ny, nx * batch, sign);
    if (rc) return rc;
    cd* twx = make_table(nx, sign);
    if (!twx) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (int64_t t = 0; t < batch * ny; ++t) {
        int64_t b = t / ny, c = t % ny;
        cd* base = (cd*)out + b * nx * ny;
        cd* col = (cd*)malloc((size_t)nx * 2 * sizeof(cd));
        if (!col) { err |= 1; continue; }
        for (int64_t i = 0; i < nx; ++i) col[nx + i] = base[i * ny + c];
        err |= c2c_one(col + nx, 1, col, nx, twx) ? 1 : 0;
        for (int64_t i = 0; i < nx; ++i) base[i * ny + c] = col[i];
        free(col);
    }
    free(twx);
    return err ? -2 : 0;
}

/* R2C: in [batch][n] doubles, out [batch][n/2+1] complex. */
int orc_r2c(const double* in, double* out, int64_t n, int64_t batch)
{
    if (n <= 0 || batch <= 0 || !in || !out) return -1;
    int64_t D = n / 2 + 1;
    if (n % 2 == 0 && n >= 2) {
        int64_t h = n / 2;
        cd* tw = make_table(h, -1);
        if (!tw) return -2;
        int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
        for (int64_t b = 0; b < batch; ++b) {
            cd* z = (cd*)malloc((size_t)h * 2 * sizeof(cd));
            if (!z) { err |= 1; continue; }
            /* pack: z[k] = x[2k] + i x[2k+1] */
            for (int64_t k = 0; k < h; ++k) {
                z[h + k].re = in[b * n + 2 * k];
                z[h + k].im = in[b * n + 2 * k + 1];
            }
            err |= c2c_one(z + h, 1, z, h, tw) ? 1 : 0;
            cd* X = (cd*)out + b * D;
            X[0].re = z[0].re + z[0].im;
            X[0].im = 0.0;
            X[h].re = z[0].re - z[0].im;
            X[h].im = 0.0;
            for (int64_t k = 1; k < h; ++k) {
                cd zk = z[k];
                cd zc = {z[h - k].re, -z[h - k].im}; /* conj(Z[h-k]) */
                double er = 0.5 * (zk.re + zc.re), ei = 0.5 * (zk.im + zc.im);
                double orr = 0.5 * (zk.im - zc.im), oi = 0.5 * (zc.re - zk.re);
                cd w = unit_root(k, n, -1);
                X[k].re = er + (w.re * orr - w.im * oi);
                X[k].im = ei + (w.re * oi + w.im * orr);
            }
            free(z);
        }
        free(tw);
        return err ? -2 : 0;
    }
    /* odd n: full complex transform of (x, 0), keep the first n/2+1 bins */
    cd* tw = make_table(n, -1);
    if (!tw) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (int64_t b = 0; b < batch; ++b) {
        cd* z = (cd*)malloc((size_t)n * 2 * sizeof(cd));
        if (!z) { err |= 1; continue; }
        for (int64_t k = 0; k < n; ++k) {
            z[n + k].re = in[b * n + k];
            z[n + k].im = 0.0;
        }
        err |= c2c_one(z + n, 1, z, n, tw) ? 1 : 0;
        memcpy((cd*)out + b * D, z, (size_t)D * sizeof(cd));
        free(z);
    }
    free(tw);
    return err ? -2 : 0;
}

/* C2R: in [batch][n/2+1] complex, out [batch][n] doubles, unscaled. */
int orc_c2r(const double* in, double* out, int64_t n, int64_t batch)
{
    if (n <= 0 || batch <= 0 || !in || !out) return -1;
    int64_t D = n / 2 + 1;
    cd* tw = make_table(n, +1);
    if (!tw) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : err)
    for (int64_t b = 0; b < batch; ++b) {
        cd* z = (cd*)malloc((size_t)n * 2 * sizeof(cd));
        if (!z) { err |= 1; continue; }
        const cd* X = (const cd*)in + b * D;
        for (int64_t k = 0; k < n; ++k) {
            cd v;
            if (k < D) {
                v = X[k];
            } else {
                int64_t i = n - k;
                v.re = X[i].re;
                v.im = -X[i].im;
            }
            z[n + k] = v;
        }
        err |= c2c_one(z + n, 1, z, n, tw) ? 1 : 0;
        for (int64_t k = 0; k < n; ++k) out[b * n + k] = z[k].re;
        free(z);
    }
    free(tw);
    return err ? -2 : 0;
}

/* Direct O(n) evaluation of selected bins of one forward/backward DFT, used
 * to cross-check the recursive oracle.  x: n complex, bins: nb indices. */
int orc_dft_bins(const double* x, int64_t n, const int64_t* bins, int64_t nb, int sign, double* out)
{
    if (n <= 0 || nb < 0 || !x || !out) return -1;
    for (int64_t t = 0; t < nb; ++t) {
        int64_t k = bins[t];
        long double sr = 0.0L, si = 0.0L;
        for (int64_t j = 0; j < n; ++j) {
            cd w = unit_root((j % n) * (k % n) % n, n, sign);
            double vr = x[2 * j], vi = x[2 * j + 1];
            sr += (long double)vr * w.re - (long double)vi * w.im;
            si += (long double)vr * w.im + (long double)vi * w.re;
        }
        out[2 * t] = (double)sr;
        out[2 * t + 1] = (double)si;
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * FP32 port of the reference arch35 Stockham path (CPU baseline only).
 * ------------------------------------------------------------------------ */
typedef struct {
    float re, im;
} cf;

typedef struct {
    int nstage;
    int radix[64];
    int64_t n;
    cf* dft[64]; /* radix x radix */
    cf* tw[64];  /* per stage: radix x prev */
} port_plan;

static int port_find_radix(int64_t n)
{
    static const int primes[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47};
    for (unsigned i = 0; i < sizeof(primes) / sizeof(primes[0]); ++i)
        if (n % primes[i] == 0) return primes[i];
    return (int)n; /* prime beyond the table: one direct stage */
}

static void port_plan_free(port_plan* p)
{
    for (int s = 0; s < p->nstage; ++s) {
        free(p->dft[s]);
        free(p->tw[s]);
    }
    p->nstage = 0;
}

static int port_plan_make(port_plan* p, int64_t n, int sign)
{
    memset(p, 0, sizeof(*p));
    p->n = n;
    int64_t rem = n, prev = 1;
    while (rem > 1) {
        int r = port_find_radix(rem);
        int s = p->nstage++;
        p->radix[s] = r;
        p->dft[s] = (cf*)malloc((size_t)r * r * sizeof(cf));
        p->tw[s] = (cf*)malloc((size_t)r * (size_t)prev * sizeof(cf));
        if (!p->dft[s] || !p->tw[s]) { port_plan_free(p); return -2; }
        for (int q = 0; q < r; ++q)
            for (int k = 0; k < r; ++k) {
                cd w = unit_root((int64_t)q * k, r, sign);
                p->dft[s][q * r + k].re = (float)w.re;
                p->dft[s][q * r + k].im = (float)w.im;
            }
        for (int k = 0; k < r; ++k)
            for (int64_t j = 0; j < prev; ++j) {
                cd w = unit_root((int64_t)k * j, prev * r, sign);
                p->tw[s][k * prev + j].re = (float)w.re;
                p->tw[s][k * prev + j].im = (float)w.im;
            }
        prev *= r;
        rem /= r;
        if (p->nstage >= 64) { port_plan_free(p); return -1; }
    }
    return 0;
}

/* One length-n transform in place on x using scratch y (both n entries). */
static void port_run(const port_plan* p, cf* x, cf* y)
{
    int64_t n = p->n, prev = 1;
    cf* a = x;
    cf* b = y;
    cf v[64];
    for (int s = 0; s < p->nstage; ++s) {
        int r = p->radix[s];
        int64_t part = n / r, len = prev * r;
        for (int64_t idx = 0; idx < part; ++idx) {
            int64_t block = idx / prev, j = idx % prev;
            for (int k = 0; k < r && k < 64; ++k) {
                cf in = a[block * prev + j + k * part];
                cf w = p->tw[s][k * prev + j];
                v[k].re = in.re * w.re - in.im * w.im;
                v[k].im = in.re * w.im + in.im * w.re;
            }
            for (int q = 0; q < r; ++q) {
                float sr = 0.f, si = 0.f;
                for (int k = 0; k < r; ++k) {
                    cf d = p->dft[s][q * r + k];
                    sr += v[k].re * d.re - v[k].im * d.im;
                    si += v[k].re * d.im + v[k].im * d.re;
                }
                b[block * len + q * prev + j].re = sr;
                b[block * len + q * prev + j].im = si;
            }
        }
        cf* t = a;
        a = b;
        b = t;
        prev = len;
    }
    if (a != x) memcpy(x, a, (size_t)n * sizeof(cf));
}

/* Float C2C port, [batch][n] interleaved floats, radices must be <= 64. */
int port_c2c(const float* in, float* out, int64_t n, int64_t batch, int sign, int nthreads)
{
    if (n <= 0 || batch <= 0) return -1;
    port_plan p;
    if (port_plan_make(&p, n, sign)) return -2;
    for (int s = 0; s < p.nstage; ++s)
        if (p.radix[s] > 64) { port_plan_free(&p); return -1; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int err = 0;
#pragma omp parallel reduction(| : err)
    {
        cf* x = (cf*)malloc((size_t)n * sizeof(cf));
        cf* y = (cf*)malloc((size_t)n * sizeof(cf));
        if (!x || !y) err |= 1;
#pragma omp for schedule(static)
        for (int64_t b = 0; b < batch; ++b) {
            if (!x || !y) continue;
            memcpy(x, in + 2 * b * n, (size_t)n * sizeof(cf));
            port_run(&p, x, y);
            memcpy(out + 2 * b * n, x, (size_t)n * sizeof(cf));
        }
        free(x);
        free(y);
    }
    port_plan_free(&p);
    return err ? -2 : 0;
}

/* Float R2C port (even n: pack, n/2 C2C, post-process; odd n: full C2C). */
int port_r2c(const float* in, float* out, int64_t n, int64_t batch, int nthreads)
{
    if (n <= 0 || batch <= 0) return -1;
    int64_t D = n / 2 + 1;
    int even = (n % 2 == 0 && n >= 2);
    int64_t h = even ? n / 2 : n;
    port_plan p;
    if (port_plan_make(&p, h, -1)) return -2;
    cf* post = (cf*)malloc((size_t)D * sizeof(cf));
    if (!post) { port_plan_free(&p); return -2; }
    for (int64_t k = 0; k < D; ++k) {
        cd w = unit_root(k, n, -1);
        post[k].re = (float)w.re;
        post[k].im = (float)w.im;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int err = 0;
#pragma omp parallel reduction(| : err)
    {
        cf* z = (cf*)malloc((size_t)h * sizeof(cf));
        cf* y = (cf*)malloc((size_t)h * sizeof(cf));
        if (!z || !y) err |= 1;
#pragma omp for schedule(static)
        for (int64_t b = 0; b < batch; ++b) {
            if (!z || !y) continue;
            const float* x = in + b * n;
            cf* X = (cf*)out + b * D;
            if (even) {
                memcpy(z, x, (size_t)n * sizeof(float));
                port_run(&p, z, y);
                X[0].re = z[0].re + z[0].im;
                X[0].im = 0.f;
                X[h].re = z[0].re - z[0].im;
                X[h].im = 0.f;
                for (int64_t k = 1; k < h; ++k) {
                    cf zk = z[k], zc = {z[h - k].re, -z[h - k].im};
                    float er = (zk.re + zc.re) / 2.f, ei = (zk.im + zc.im) / 2.f;
                    float orr = (zk.im - zc.im) / 2.f, oi = (zc.re - zk.re) / 2.f;
                    cf w = post[k];
                    X[k].re = er + (w.re * orr - w.im * oi);
                    X[k].im = ei + (w.re * oi + w.im * orr);
                }
            } else {
                for (int64_t k = 0; k < n; ++k) {
                    z[k].re = x[k];
                    z[k].im = 0.f;
                }
                port_run(&p, z, y);
                memcpy(X, z, (size_t)D * sizeof(cf));
            }
        }
        free(z);
        free(y);
    }
    free(post);
    port_plan_free(&p);
    return err ? -2 : 0;
}

/* Float C2R port: Hermitian expansion, full n-point inverse, real part. */
int port_c2r(const float* in, float* out, int64_t n, int64_t batch, int nthreads)
{
    if (n <= 0 || batch <= 0) return -1;
    int64_t D = n / 2 + 1;
    port_plan p;
    if (port_plan_make(&p, n, +1)) return -2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int err = 0;
#pragma omp parallel reduction(| : err)
    {
        cf* z = (cf*)malloc((size_t)n * sizeof(cf));
        cf* y = (cf*)malloc((size_t)n * sizeof(cf));
        if (!z || !y) err |= 1;
#pragma omp for schedule(static)
        for (int64_t b = 0; b < batch; ++b) {
            if (!z || !y) continue;
            const cf* X = (const cf*)in + b * D;
            for (int64_t k = 0; k < n; ++k) {
                if (k < D) {
                    z[k] = X[k];
                } else {
                    z[k].re = X[n - k].re;
                    z[k].im = -X[n - k].im;
                }
            }
            port_run(&p, z, y);
            for (int64_t k = 0; k < n; ++k) out[b * n + k] = z[k].re;
        }
        free(z);
        free(y);
    }
    port_plan_free(&p);
    return err ? -2 : 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
