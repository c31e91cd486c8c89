// dfft.cu - double-precision (Z2Z / D2Z / Z2D) transforms.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, so a
// double-precision FFT is bound by arithmetic, not by HBM: the passes here
// are plain global-memory-to-global-memory Stockham passes (one radix-R
// butterfly per thread, the same compile-time butterflies as the FP32
// kernels instantiated on double2), not the shared-memory pipelines of the
// FP32 path.  A transform of length n = R_1 * ... * R_k is k launches; the
// planner routes them through two workspaces (a pass never writes the buffer
// it reads).  Twiddles come from a per-plan table W_n^m (m < n) generated in
// FP64 on the GPU.
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterfly.cuh"
#include "kernel_args.h"
#include "pdl.cuh"

namespace gfft {
namespace {

__device__ __forceinline__ int64_t dbase(int64_t t, int64_t split, int64_t hi, int64_t lo)
{
    return (t / split) * hi + (t % split) * lo;
}

template <int R>
__global__ void __launch_bounds__(256) dpass_kernel(const __grid_constant__ DPassArgs a)
{
    pdl_wait();
    const int n = a.n;
    const int nbf = n / R;
    const int64_t total = a.ntf * nbf;
    const double2* tw = static_cast<const double2*>(a.tw);
    const int step = n / (a.ns * R);  // table stride of W_{ns*R}
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int64_t t;
        int j;
        if (a.t_fast) {
            t = idx % a.ntf;
            j = (int)(idx / a.ntf);
        } else {
            j = (int)(idx % nbf);
            t = idx / nbf;
        }
        const int64_t ib = dbase(t, a.in_split, a.in_hi, a.in_lo);
        const int64_t ob = dbase(t, a.out_split, a.out_hi, a.out_lo);
        double2 v[R];
        if (a.io & DIO_REAL_IN) {
            const double* x = static_cast<const double*>(a.in) + ib;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[r] = make_double2(x[(int64_t)(j + r * nbf) * a.in_stride], 0.0);
            });
        } else if (a.io & DIO_HERM_IN) {
            // conj of the Hermitian extension: conj(X[i]) for i <= n/2, X[n-i] above
            const double2* x = static_cast<const double2*>(a.in) + ib;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const int i = j + r * nbf;
                v[r] = (2 * i <= n) ? cconj(x[(int64_t)i * a.in_stride]) : x[(int64_t)(n - i) * a.in_stride];
            });
        } else if (a.io & DIO_PAIR_IN) {
            const double* x = static_cast<const double*>(a.in) + 2 * ib;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const int64_t e = 2 * (int64_t)(j + r * nbf) * a.in_stride;
                v[r] = make_double2(x[e], a.conj_in ? -x[e + 1] : x[e + 1]);
            });
        } else {
            const double2* x = static_cast<const double2*>(a.in) + ib;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const double2 e = x[(int64_t)(j + r * nbf) * a.in_stride];
                v[r] = a.conj_in ? cconj(e) : e;
            });
        }
        const int k = j % a.ns;
        if (a.ns > 1) {
            sfor<R - 1>([&](auto rr) {
                constexpr int r = decltype(rr)::value + 1;
                v[r] = cmul(v[r], tw[k * r * step]);
            });
        }
        DFT<R>::run(v);
        const int o0 = (j - k) * R + k;  // (j/ns)*ns*R + j%ns
        if (a.io & DIO_REAL_OUT) {
            double* y = static_cast<double*>(a.out) + ob;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                y[(int64_t)(o0 + r * a.ns) * a.out_stride] = v[r].x * a.scale;
            });
        } else if (a.io & DIO_PAIR_OUT) {
            double* y = static_cast<double*>(a.out) + 2 * ob;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                double2 e = a.conj_out ? cconj(v[r]) : v[r];
                if (a.scale != 1.0) e = cscale(e, a.scale);
                const int64_t o = 2 * (int64_t)(o0 + r * a.ns) * a.out_stride;
                y[o] = e.x;
                y[o + 1] = e.y;
            });
        } else {
            double2* y = static_cast<double2*>(a.out) + ob;
            const bool half = (a.io & DIO_HALF_OUT) != 0;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const int o = o0 + r * a.ns;
                if (!half || 2 * o <= n) {
                    double2 e = a.conj_out ? cconj(v[r]) : v[r];
                    if (a.scale != 1.0) e = cscale(e, a.scale);
                    y[(int64_t)o * a.out_stride] = e;
                }
            });
        }
    }
}

// Even N = 2L, transform t, pair (k, L - k) for k = 0..L/2 per thread.
// D2Z post-process: Z (L values) -> X (L + 1 bins),
//   E = (Z[k] + conj Z[L-k])/2, O = (Z[k] - conj Z[L-k])/(2i),
//   X[k] = E + W_N^k O, X[L-k] = conj(E - W_N^k O),
//   X[0] = Re Z0 + Im Z0, X[L] = Re Z0 - Im Z0;
// Z2D pre-process: X (L + 1 bins) -> Z' (L values), stored conjugated so
// that a forward transform and a conjugated store give the backward one,
//   E = X[k] + conj X[L-k], O = (X[k] - conj X[L-k]) * conj W_N^k,
//   Z'[k] = conj(E + iO), Z'[L-k] = conj(conj E + i conj O),
//   Z'[0] = (Re X0 + Re XL, -(Re X0 - Re XL)) (imaginary parts of DC and
//   Nyquist ignored).
__global__ void __launch_bounds__(256) dreal_kernel(const __grid_constant__ DPassArgs a)
{
    pdl_wait();
    const int L = a.n / 2;
    const int np = L / 2 + 1;
    const int64_t total = a.ntf * np;
    const double2* tw = static_cast<const double2*>(a.tw);
    const bool post = (a.io & DIO_R2C_POST) != 0;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % np);
        const int64_t t = idx / np;
        const double2* x = static_cast<const double2*>(a.in) + t * a.in_hi;
        double2* y = static_cast<double2*>(a.out) + t * a.out_hi;
        if (post) {
            const double sc = a.scale;
            if (k == 0) {
                const double2 z0 = x[0];
                y[0] = make_double2((z0.x + z0.y) * sc, 0.0);
                y[L] = make_double2((z0.x - z0.y) * sc, 0.0);
                continue;
            }
            const double2 zk = x[k], zc = cconj(x[L - k]);
            const double2 e = make_double2(0.5 * (zk.x + zc.x), 0.5 * (zk.y + zc.y));
            const double2 o = make_double2(0.5 * (zk.y - zc.y), 0.5 * (zc.x - zk.x));
            const double2 wo = cmul(tw[k], o);
            y[k] = cscale(cadd(e, wo), sc);
            if (L - k != k) y[L - k] = cscale(cconj(csub(e, wo)), sc);
        } else {
            if (k == 0) {
                const double x0 = x[0].x, xl = x[L].x;
                y[0] = make_double2(x0 + xl, -(x0 - xl));
                continue;
            }
            const double2 xa = x[k], xb = cconj(x[L - k]);
            const double2 e = cadd(xa, xb);
            const double2 o = cmulc(csub(xa, xb), tw[k]);
            y[k] = cconj(make_double2(e.x - o.y, e.y + o.x));
            if (L - k != k) y[L - k] = cconj(make_double2(e.x + o.y, -e.y + o.x));
        }
    }
}

__global__ void dtw_kernel(double2* tab, long long n)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += (long long)gridDim.x * blockDim.x) {
        // angle 2*pi*m/n as a multiple of pi, reduced exactly to [0, 2)
        double s, c;
        sincospi((double)(2 * m) / (double)n, &s, &c);
        tab[m] = make_double2(c, -s);
    }
}

template <int R>
int launch_r(const DPassArgs* a, cudaStream_t st)
{
    const int64_t total = a->ntf * (a->n / R);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return (int)cudaErrorInvalidValue;
    const int64_t blocks = (total + 255) / 256;
    const int64_t grid = blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8;
    return (int)launch_pdl(dpass_kernel<R>, dim3((unsigned)(grid > 0 ? grid : 1)), dim3(256), 0, st, *a);
}

}  // namespace
}  // namespace gfft

extern "C" int gfft_launch_dpass(const gfft::DPassArgs* a, void* stream)
{
    using namespace gfft;
    if (a->n < 1 || a->radix < 1 || a->n % a->radix || a->ns < 1 || (a->n / a->radix) % a->ns || a->ntf < 1 ||
        a->in_split < 1 || a->out_split < 1)
        return (int)cudaErrorInvalidValue;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (a->io & (DIO_R2C_POST | DIO_C2R_PRE)) {
        if (a->n % 2) return (int)cudaErrorInvalidValue;
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return (int)cudaErrorInvalidValue;
        const int64_t total = a->ntf * (a->n / 4 + 1);
        const int64_t blocks = (total + 255) / 256;
        const int64_t grid = blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8;
        return (int)launch_pdl(dreal_kernel, dim3((unsigned)(grid > 0 ? grid : 1)), dim3(256), 0, st, *a);
    }
    switch (a->radix) {
#define GFFT_DR(R) \
    case R: return launch_r<R>(a, st);
        GFFT_DR(1) GFFT_DR(2) GFFT_DR(3) GFFT_DR(4) GFFT_DR(5) GFFT_DR(6) GFFT_DR(7) GFFT_DR(8) GFFT_DR(9)
        GFFT_DR(10) GFFT_DR(11) GFFT_DR(12) GFFT_DR(13) GFFT_DR(14) GFFT_DR(15) GFFT_DR(16) GFFT_DR(17)
        GFFT_DR(19) GFFT_DR(23) GFFT_DR(29) GFFT_DR(31) GFFT_DR(37) GFFT_DR(41) GFFT_DR(43) GFFT_DR(47)
#undef GFFT_DR
    default: return (int)cudaErrorInvalidValue;
    }
}

extern "C" int gfft_gen_dtwiddles(void* table, long long n, void* stream)
{
    if (!table || n < 1) return (int)cudaErrorInvalidValue;
    const long long blocks = (n + 255) / 256;
    gfft::dtw_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<double2*>(table), n);
    return (int)cudaGetLastError();
}
