// fft_misc.cu - launcher dispatch, FP64 twiddle generation and the
// stand-alone even/odd packing kernel.
#include <cuda_runtime.h>
#include <math.h>

#include "codelet_list.h"
#include "launch_common.cuh"

namespace gfft {

// out[i] = exp(-2*pi*i*f(i)/M) evaluated in FP64 and rounded to FP32.  The
// integer f(i) is reduced modulo M before the division so the argument of
// sincospi stays in [0, 2) with full double precision.
__global__ void twiddle_kernel(float2* __restrict__ out, TwSeg seg)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < seg.count; i += stride) {
        int64_t m;
        if (seg.kind == 2) {
            const int64_t ns = seg.R_or_mult;
            m = ((i / ns) * (i % ns)) % seg.M;
        } else {
            m = (int64_t)(((unsigned __int128)i * (unsigned __int128)seg.R_or_mult) % (unsigned __int128)seg.M);
        }
        double s, c;
        sincospi(-2.0 * (double)m / (double)seg.M, &s, &c);
        out[seg.offset + i] = make_float2((float)c, (float)s);
    }
}

// Even/odd packing for real transforms whose half length does not fit one
// CTA (see the fused versions in stockham.cuh for the formulas).
__global__ void pack_kernel(PackArgs a)
{
    pdl_wait();
    const int L = a.L;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > (L >> 1)) return;
    for (int64_t t = blockIdx.y; t < a.ntf; t += gridDim.y) {
    const float2* in = reinterpret_cast<const float2*>(a.in) + t * a.in_dist;
    float2* out = reinterpret_cast<float2*>(a.out) + t * a.out_dist;
    const float2* post = reinterpret_cast<const float2*>(a.post_tw);
    const float sc = a.scale;
    if (!a.c2r) {
        if (k == 0) {
            const float2 z0 = in[0];
            out[0] = make_float2((z0.x + z0.y) * sc, 0.f);
            out[L] = make_float2((z0.x - z0.y) * sc, 0.f);
            continue;
        }
        const float2 zk = in[k], zc = cconj(in[L - k]);
        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
        const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
        const float2 wo = cmul(post[k], o);
        const float s2 = a.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
        out[k] = cscale(cadd(e, wo), s2);
        if (L - k != k) out[L - k] = cscale(cconj(csub(e, wo)), s2);
    } else {
        if (k == 0) {
            const float x0 = in[0].x, xl = in[L].x;
            out[0] = make_float2(x0 + xl, -(x0 - xl));
            continue;
        }
        float2 x = in[k], y = in[L - k];
        if (a.weight == WEIGHT_LOAD_HALF) {
            x = cscale(x, 0.5f);
            y = cscale(y, 0.5f);
        }
        const float2 w = post[k];
        const float2 yc = cconj(y);
        const float2 e = cadd(x, yc);
        const float2 o = cmulc(csub(x, yc), w);
        out[k] = cconj(make_float2(e.x - o.y, e.y + o.x));
        if (L - k != k) out[L - k] = cconj(make_float2(e.x + o.y, -e.y + o.x));
    }
    }
}

}  // namespace gfft

using namespace gfft;

extern "C" int gfft_launch_row(const RowArgs* a, void* stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (a->codelet) {
    case -1: break;
#define GFFT_CASE_ROW(ID, ...) \
    case ID: return launch_codelet_##ID(a, st);
        GFFT_CODELETS(GFFT_CASE_ROW)
#undef GFFT_CASE_ROW
    default: return (int)cudaErrorInvalidValue;
    }
    switch (a->ip.rmax) {
    case 16: return launch_row_r16(a, st);
    case 47: return launch_row_r47(a, st);
    default: return (int)cudaErrorInvalidValue;
    }
}

extern "C" int gfft_launch_col(const ColArgs* a, void* stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (a->codelet) {
    case -1: break;
#define GFFT_CASE_COL(ID, ...) \
    case ID: return launch_coltile_##ID(a, st);
        GFFT_CODELETS(GFFT_CASE_COL)
#undef GFFT_CASE_COL
    default: return (int)cudaErrorInvalidValue;
    }
    switch (a->ip.rmax) {
    case 16: return launch_col_r16(a, st);
    case 47: return launch_col_r47(a, st);
    default: return (int)cudaErrorInvalidValue;
    }
}

extern "C" int gfft_kernel_max_threads(int rmax)
{
    return rmax == 16 ? kernel_max_threads<16>() : (rmax == 47 ? kernel_max_threads<47>() : 0);
}

extern "C" int gfft_launch_pack(const PackArgs* a, void* stream)
{
    if (a->ntf <= 0 || a->L < 1) return (int)cudaErrorInvalidValue;
    const int n = (a->L >> 1) + 1;
    dim3 grid((n + 255) / 256, (unsigned)(a->ntf < 65535 ? a->ntf : 65535));
    return (int)launch_pdl(pack_kernel, grid, dim3(256), 0, static_cast<cudaStream_t>(stream), *a);
}

extern "C" int gfft_gen_twiddles(void* table, const TwSeg* segs, int nseg, void* stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int i = 0; i < nseg; ++i) {
        if (segs[i].count <= 0) continue;
        if (segs[i].kind == 3) {
            const int rc = gfft_tc_gen_bmat(static_cast<float2*>(table) + segs[i].offset, (int)segs[i].M,
                                            (int)segs[i].R_or_mult, stream);
            if (rc != 0) return rc;
            continue;
        }
        const int64_t blocks64 = (segs[i].count + 255) / 256;
        const unsigned blocks = (unsigned)(blocks64 > 4096 ? 4096 : blocks64);
        twiddle_kernel<<<blocks, 256, 0, st>>>(static_cast<float2*>(table), segs[i]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

extern "C" int gfft_codelet_lookup(int L, int* nthr, int* radices, int* nradix)
{
    int maxt = 0;
    return gfft_codelet_lookup2(L, nthr, radices, nradix, &maxt);
}

extern "C" int gfft_codelet_find(int L, int variant)
{
    int k = 0;
#define GFFT_FIND(ID, MT, MB, LL, NT, ...) \
    if (L == LL && k++ == variant) return ID;
    GFFT_CODELETS(GFFT_FIND)
#undef GFFT_FIND
    return -1;
}

extern "C" int gfft_codelet_info(int id, int* L, int* nthr, int* radices, int* nradix, int* maxt, int* minb)
{
#define GFFT_INFO(ID, MT, MB, LL, NT, ...)                     \
    if (id == ID) {                                            \
        const int r[] = {__VA_ARGS__};                         \
        *L = LL;                                               \
        *nthr = NT;                                            \
        *maxt = MT;                                            \
        *minb = MB;                                            \
        *nradix = (int)(sizeof(r) / sizeof(r[0]));             \
        for (int i = 0; i < *nradix; ++i) radices[i] = r[i];   \
        return 0;                                              \
    }
    GFFT_CODELETS(GFFT_INFO)
#undef GFFT_INFO
    return -1;
}

extern "C" int gfft_codelet_lookup2(int L, int* nthr, int* radices, int* nradix, int* maxt)
{
#define GFFT_LOOKUP(ID, MT, MB, LL, NT, ...)                           \
    if (L == LL) {                                             \
        const int r[] = {__VA_ARGS__};                         \
        *nthr = NT;                                            \
        *maxt = MT;                                            \
        *nradix = (int)(sizeof(r) / sizeof(r[0]));             \
        for (int i = 0; i < *nradix; ++i) radices[i] = r[i];   \
        return ID;                                             \
    }
    GFFT_CODELETS(GFFT_LOOKUP)
#undef GFFT_LOOKUP
    return -1;
}
