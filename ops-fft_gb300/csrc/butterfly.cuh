// butterfly.cuh - in-register DFT butterflies for the Stockham kernels.
//
// DFT<R>::run(v) replaces v[0..R) by its forward (exp(-2*pi*i*k*n/R)) DFT in
// natural order.  Every twiddle inside a butterfly is a compile-time constant
// computed by our own constexpr sin/cos (a Taylor series in double after an
// exact integer octant reduction), so the generated code holds immediates
// only.  Backward transforms reuse the forward butterflies through
// conj(DFT(conj(x))), applied by the kernels at load and store.
//
// Radix families:
//   2, 3, 4, 5, 7          hand-derived minimal-operation forms
//   odd primes p (11..47)  symmetric-pair form: for k = 1..(p-1)/2,
//                          X_k, X_{p-k} = x0 + sum_j c_jk A_j -/+ i sum_j s_jk B_j
//                          with A_j = x_j + x_{p-j}, B_j = x_j - x_{p-j}
//   composite R = A*B      with gcd(A, B) = 1 (6, 10, 12, 14, 15, 18, 20, ...):
//                          the prime-factor (Good-Thomas) split, no
//                          inter-stage twiddles: x[(B*n1 + A*n2) mod R]
//                          through B-point then A-point DFTs, bin k1, k2
//                          stored at the k with k = k1 mod A, k = k2 mod B;
//                          otherwise (8, 9, 16, ...) one decimation-in-time
//                          split (A-point over B-point) with constant
//                          inter-stage twiddles W_R^{a*k1}
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

#ifndef GFFT_HD
#define GFFT_HD __host__ __device__ __forceinline__
#endif

namespace gfft {

// ----------------------------------------------------------- static loops
template <class F, int... Is>
GFFT_HD void sfor_impl(F&& f, std::integer_sequence<int, Is...>)
{
    (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
GFFT_HD void sfor(F&& f)
{
    sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// ------------------------------------------------- compile-time unit roots
constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double taylor_sin(double x)
{
    double term = x, sum = x;
    const double x2 = x * x;
    for (int k = 1; k < 16; ++k) {
        term *= -x2 / double((2 * k) * (2 * k + 1));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double taylor_cos(double x)
{
    double term = 1.0, sum = 1.0;
    const double x2 = x * x;
    for (int k = 1; k < 16; ++k) {
        term *= -x2 / double((2 * k - 1) * (2 * k));
        sum += term;
    }
    return sum;
}

struct Root {
    double c, s;  // cos and sin of the positive angle 2*pi*num/den
};

// cos/sin of 2*pi*num/den with the angle reduced exactly to one octant.
__host__ __device__ constexpr Root unit_root(long long num, long long den)
{
    long long m = num % den;
    if (m < 0) m += den;
    const long long e = 8 * m;
    const int oct = int(e / den);
    const long long rem = e - (long long)oct * den;
    const double a = double(rem) / double(den) * (kPi / 4.0);
    const double ca = taylor_cos(a), sa = taylor_sin(a);
    const double cb = taylor_cos(kPi / 4.0 - a), sb = taylor_sin(kPi / 4.0 - a);
    switch (oct & 7) {
    case 0: return {ca, sa};
    case 1: return {sb, cb};
    case 2: return {-sa, ca};
    case 3: return {-cb, sb};
    case 4: return {-ca, -sa};
    case 5: return {-sb, -cb};
    case 6: return {sa, -ca};
    default: return {cb, -sb};
    }
}

// Forward twiddle W_R^E = exp(-2*pi*i*E/R) as float components.
template <int R, int E>
struct W {
    static constexpr Root r = unit_root(E, R);
    static constexpr float re = float(r.c);
    static constexpr float im = float(-r.s);
};

// ------------------------------------------------------ complex helpers
// On sm_100+ device code the helpers use the paired FP32 instructions
// (one FADD2/FMUL2/FFMA2 per complex op instead of two scalar ops).  Each
// lane of a paired op rounds exactly like the scalar op it replaces, so
// results are bit-identical to the scalar host forms below.
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000) && !defined(GFFT_SCALAR_COMPLEX)
#define GFFT_PAIRED 1
#endif

GFFT_HD float2 cadd(float2 a, float2 b)
{
#ifdef GFFT_PAIRED
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
GFFT_HD float2 csub(float2 a, float2 b)
{
#ifdef GFFT_PAIRED
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
GFFT_HD float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
GFFT_HD float2 cscale(float2 a, float s)
{
#ifdef GFFT_PAIRED
    return __fmul2_rn(a, make_float2(s, s));
#else
    return make_float2(a.x * s, a.y * s);
#endif
}
// (re, im) = (a.x*b.x - a.y*b.y, a.x*b.y + a.y*b.x), the products a.y*b
// rounded first and the a.x*b terms fused.
GFFT_HD float2 cmul(float2 a, float2 b)
{
#ifdef GFFT_PAIRED
    const float2 t = __fmul2_rn(make_float2(a.y, a.y), make_float2(b.y, b.x));
    return __ffma2_rn(make_float2(a.x, a.x), b, make_float2(-t.x, t.y));
#else
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
#endif
}
// a * conj(b) = (a.x*b.x + a.y*b.y, a.y*b.x - a.x*b.y)
GFFT_HD float2 cmulc(float2 a, float2 b)
{
#ifdef GFFT_PAIRED
    const float2 t = __fmul2_rn(make_float2(a.y, a.x), make_float2(b.y, b.y));
    return __ffma2_rn(make_float2(a.x, a.y), make_float2(b.x, b.x), make_float2(t.x, -t.y));
#else
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
#endif
}
// acc + s * a per component (fused).
GFFT_HD float2 sfma(float s, float2 a, float2 acc)
{
#ifdef GFFT_PAIRED
    return __ffma2_rn(make_float2(s, s), a, acc);
#else
    return make_float2(fmaf(s, a.x, acc.x), fmaf(s, a.y, acc.y));
#endif
}
// a * b per component.
GFFT_HD float2 pmul(float2 a, float2 b)
{
#ifdef GFFT_PAIRED
    return __fmul2_rn(a, b);
#else
    return make_float2(a.x * b.x, a.y * b.y);
#endif
}
// (a + b) * h per component (the odd multiples of pi/4 rotations).
GFFT_HD float2 sum_scale(float2 a, float2 b, float h) { return cscale(cadd(a, b), h); }
GFFT_HD float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // * (-i)
GFFT_HD float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }  // * (+i)

// FP64 complex helpers (double-precision transforms): scalar double ops,
// fused where the FP32 forms are.
GFFT_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
GFFT_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
GFFT_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
GFFT_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
GFFT_HD double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
GFFT_HD double2 cmulc(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
GFFT_HD double2 sfma(double s, double2 a, double2 acc) { return make_double2(fma(s, a.x, acc.x), fma(s, a.y, acc.y)); }
GFFT_HD double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
GFFT_HD double2 sum_scale(double2 a, double2 b, double h) { return cscale(cadd(a, b), h); }
GFFT_HD double2 mul_mi(double2 a) { return make_double2(a.y, -a.x); }
GFFT_HD double2 mul_pi(double2 a) { return make_double2(-a.y, a.x); }

// Component type and constructor of a complex vector type.
template <class C>
struct CT;
template <>
struct CT<float2> {
    using S = float;
    GFFT_HD static float2 make(float a, float b) { return make_float2(a, b); }
};
template <>
struct CT<double2> {
    using S = double;
    GFFT_HD static double2 make(double a, double b) { return make_double2(a, b); }
};

// x * W_R^E with the trivial angles folded at compile time.
template <int R, int E, class C>
GFFT_HD C twc(C x)
{
    using T = CT<C>;
    using S = typename T::S;
    constexpr int e = ((E % R) + R) % R;
    constexpr S h = S(W<8, 1>::r.c);  // cos(pi/4)
    if constexpr (e == 0) {
        return x;
    } else if constexpr (2 * e == R) {
        return T::make(-x.x, -x.y);
    } else if constexpr (4 * e == R) {
        return mul_mi(x);
    } else if constexpr (4 * e == 3 * R) {
        return mul_pi(x);
    } else if constexpr (8 * e == R) {
        return sum_scale(T::make(x.x, x.y), T::make(x.y, -x.x), h);
    } else if constexpr (8 * e == 3 * R) {
        return sum_scale(T::make(x.y, -x.x), T::make(-x.x, -x.y), h);
    } else if constexpr (8 * e == 5 * R) {
        return sum_scale(T::make(-x.x, x.x), T::make(-x.y, -x.y), h);
    } else if constexpr (8 * e == 7 * R) {
        return sum_scale(T::make(x.x, x.x), T::make(-x.y, x.y), h);
    } else {
        return cmul(x, T::make(S(W<R, e>::r.c), S(-W<R, e>::r.s)));
    }
}

// --------------------------------------------------------- radix tables
__host__ __device__ constexpr int smallest_factor(int n)
{
    if (n % 4 == 0 && n > 4) return 4;
    for (int f = 2; f * f <= n; ++f)
        if (n % f == 0) return f;
    return n;
}
__host__ __device__ constexpr bool is_prime(int n)
{
    if (n < 2) return false;
    for (int f = 2; f * f <= n; ++f)
        if (n % f == 0) return false;
    return true;
}
__host__ __device__ constexpr int gcd_c(int a, int b) { return b == 0 ? a : gcd_c(b, a % b); }
// x with (a * x) % m == 1 (a, m coprime, m >= 2); 0 for m == 1
__host__ __device__ constexpr int inv_mod(int a, int m)
{
    for (int x = 1; x < m; ++x)
        if ((a * x) % m == 1) return x;
    return 0;
}
// composite radices whose smallest-factor split is coprime take the
// prime-factor form
__host__ __device__ constexpr bool pfa_split(int R)
{
    return R > 4 && !is_prime(R) && gcd_c(smallest_factor(R), R / smallest_factor(R)) == 1;
}

// DFT<R>::run(v) on float2 (FP32 kernels) or double2 (FP64 transforms).
template <int R, class Enable = void>
struct DFT;

template <>
struct DFT<1> {
    template <class C>
    GFFT_HD static void run(C*)
    {
    }
};

template <>
struct DFT<2> {
    template <class C>
    GFFT_HD static void run(C* v)
    {
        const C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <>
struct DFT<3> {
    template <class C>
    GFFT_HD static void run(C* v)
    {
        using T = CT<C>;
        using S = typename T::S;
        constexpr S s3 = S(0.86602540378443864676372317075294);  // sin(2pi/3)
        const C t1 = cadd(v[1], v[2]);
        const C t2 = sfma(S(-0.5), t1, v[0]);
        const C d = csub(v[1], v[2]);
        const C t3 = pmul(T::make(s3, -s3), T::make(d.y, d.x));  // -i*s3*(v1-v2)
        v[0] = cadd(v[0], t1);
        v[1] = cadd(t2, t3);
        v[2] = csub(t2, t3);
    }
};

template <>
struct DFT<4> {
    template <class C>
    GFFT_HD static void run(C* v)
    {
        const C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        const C c = cadd(v[1], v[3]), d = mul_mi(csub(v[1], v[3]));
        v[0] = cadd(a, c);
        v[2] = csub(a, c);
        v[1] = cadd(b, d);
        v[3] = csub(b, d);
    }
};

// Odd primes >= 5: symmetric-pair evaluation.
template <int P>
struct DFT<P, std::enable_if_t<(P >= 5) && is_prime(P)>> {
    template <class C>
    GFFT_HD static void run(C* v)
    {
        using T = CT<C>;
        using S = typename T::S;
        constexpr int H = (P - 1) / 2;
        C A[H], B[H];
        C sum = v[0];
        sfor<H>([&](auto jj) {
            constexpr int j = decltype(jj)::value + 1;
            A[j - 1] = cadd(v[j], v[P - j]);
            B[j - 1] = csub(v[j], v[P - j]);
            sum = cadd(sum, A[j - 1]);
        });
        const C x0 = v[0];
        v[0] = sum;
        sfor<H>([&](auto kk) {
            constexpr int k = decltype(kk)::value + 1;
            C re = x0;                       // x0 + sum c*A
            C im = T::make(S(0), S(0));      // sum s*B
            sfor<H>([&](auto jj) {
                constexpr int j = decltype(jj)::value + 1;
                constexpr Root rt = unit_root((long long)j * k, P);
                constexpr S c = S(rt.c), s = S(rt.s);
                re = sfma(c, A[j - 1], re);
                im = sfma(s, B[j - 1], im);
            });
            // X_k = re - i*im ; X_{P-k} = re + i*im
            v[k] = cadd(re, T::make(im.y, -im.x));
            v[P - k] = cadd(re, T::make(-im.y, im.x));
        });
    }
};

// Composite radices R = A * B with gcd(A, B) = 1: prime-factor split.
template <int R>
struct DFT<R, std::enable_if_t<pfa_split(R)>> {
    static constexpr int A = smallest_factor(R);
    static constexpr int B = R / A;
    static constexpr int IA = inv_mod(B % A, A);  // B^-1 mod A
    static constexpr int IB = inv_mod(A % B, B);  // A^-1 mod B
    template <class C>
    GFFT_HD static void run(C* v)
    {
        C t[R];
        sfor<A>([&](auto aa) {
            constexpr int n1 = decltype(aa)::value;
            C u[B];
            sfor<B>([&](auto mm) {
                constexpr int n2 = decltype(mm)::value;
                u[n2] = v[(B * n1 + A * n2) % R];
            });
            DFT<B>::run(u);
            sfor<B>([&](auto kk) {
                constexpr int k2 = decltype(kk)::value;
                t[n1 * B + k2] = u[k2];
            });
        });
        sfor<B>([&](auto kk) {
            constexpr int k2 = decltype(kk)::value;
            C w[A];
            sfor<A>([&](auto aa) {
                constexpr int n1 = decltype(aa)::value;
                w[n1] = t[n1 * B + k2];
            });
            DFT<A>::run(w);
            sfor<A>([&](auto qq) {
                constexpr int k1 = decltype(qq)::value;
                // k = k1 (mod A), k = k2 (mod B)
                v[(B * ((IA * k1) % A) + A * ((IB * k2) % B)) % R] = w[k1];
            });
        });
    }
};

// Other composite radices: R = A * B, decimation in time.
template <int R>
struct DFT<R, std::enable_if_t<(R > 4) && !is_prime(R) && !pfa_split(R)>> {
    static constexpr int A = smallest_factor(R);
    static constexpr int B = R / A;
    template <class C>
    GFFT_HD static void run(C* v)
    {
        C t[R];
        sfor<A>([&](auto aa) {
            constexpr int a = decltype(aa)::value;
            C u[B];
            sfor<B>([&](auto mm) {
                constexpr int m = decltype(mm)::value;
                u[m] = v[a + A * m];
            });
            DFT<B>::run(u);
            sfor<B>([&](auto kk) {
                constexpr int k1 = decltype(kk)::value;
                t[a * B + k1] = twc<R, a * k1>(u[k1]);
            });
        });
        sfor<B>([&](auto kk) {
            constexpr int k1 = decltype(kk)::value;
            C w[A];
            sfor<A>([&](auto aa) {
                constexpr int a = decltype(aa)::value;
                w[a] = t[a * B + k1];
            });
            DFT<A>::run(w);
            sfor<A>([&](auto qq) {
                constexpr int k2 = decltype(qq)::value;
                v[k1 + B * k2] = w[k2];
            });
        });
    }
};

}  // namespace gfft
