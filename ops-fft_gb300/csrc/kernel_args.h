// kernel_args.h - argument blocks shared by the host planner (lib/) and the
// CUDA kernels (csrc/).  Plain C++ with fixed-width fields only, so the host
// side compiles without CUDA headers.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace gfft {

constexpr int kMaxPass = 12;        // on-chip Stockham passes per transform
constexpr int kMaxSmemBytes = 227 * 1024;

// One on-chip Stockham pass: radix R after a product `ns` of earlier radices.
// Butterfly j reads x[j + r*L/R] and writes y[(j/ns)*ns*R + j%ns + r*ns]
// after multiplying input r by W_{ns*R}^{(j%ns)*r}, read from the table at
// tw_off, entry r*ns + j%ns.
struct PassDesc {
    int32_t radix;
    int32_t ns;
    uint32_t ns_magic;  // ceil(2^32/ns): j/ns == umulhi(j, magic) for j, ns < 2^16
    int32_t tw_off;     // float2 offset of this pass's table, -1 when ns == 1
};

// How the on-chip transform of length L is executed.
struct InnerPlan {
    int32_t L;
    int32_t npass;
    int32_t rmax;   // largest radix, selects the kernel instantiation (16 or 47)
    int32_t nthr;   // threads cooperating on one transform
    PassDesc pass[kMaxPass];
};

enum IoMode : int32_t {
    IO_C2C = 0,       // complex in, complex out
    IO_R2C_EVEN = 1,  // real in viewed as L=N/2 complex, fused even/odd post-process
    IO_C2R_EVEN = 2,  // N/2+1 bins in, fused pre-process, real out viewed as complex
    IO_R2C_ODD = 3,   // real in, full N-point transform, first N/2+1 bins out
    IO_C2R_ODD = 4,   // Hermitian-expanded load, full N-point transform, real part out
};

enum WeightMode : int32_t {
    WEIGHT_NONE = 0,
    WEIGHT_STORE_X2 = 1,   // multiply interior output bins by 2 (C2R adjoint)
    WEIGHT_LOAD_HALF = 2,  // multiply interior input bins by 1/2 (R2C adjoint)
};

// Contiguous transforms, one on-chip transform per batch item.  The row
// kernel is persistent: CTA b handles tiles b, b + grid, ... of `tfpc`
// consecutive transforms; the raw input of upcoming tiles is prefetched into
// `nstage` shared stage buffers with bulk asynchronous copies.
struct RowArgs {
    InnerPlan ip;
    const void* tw;       // float2 twiddle blob (device)
    const void* post_tw;  // float2 W_N^k for k <= L/2 (even R2C/C2R), N = 2L
    const void* in;
    void* out;
    int* err;             // device error word (bounded waits that timed out)
    int64_t ntf;       // number of transforms
    int64_t in_dist;   // distance between transforms, in elements of the input type
    int64_t out_dist;  // same for the output
    int32_t tfpc;      // transforms per tile (per CTA iteration)
    int32_t lpad;      // float2 pitch of one shared work buffer
    int32_t nbuf;      // shared work buffers per transform (1 or 2)
    int32_t io_mode;
    int32_t conj_in;   // conjugate on load (backward transforms)
    int32_t conj_out;  // conjugate on store
    int32_t weight;
    int32_t nreal;     // N for the real-data modes
    int32_t staged;    // write results through shared memory (small transforms)
    float scale;
    int32_t nstage;    // input stage buffers
    int32_t pshift;    // shared padding: index i is stored at i + (i >> pshift)
    int32_t in_esize;  // bytes per input element: 4 (real) or 8 (complex)
    int32_t tw_lo;     // first float2 of the pass tables in the blob
    int32_t tw_cnt;    // float2 entries of the pass tables copied to shared memory
    int32_t post_cnt;  // post-process twiddles copied to shared memory
    int32_t stage_bytes;
    int32_t smem_tw, smem_post, smem_stage, smem_work, smem_bytes;  // byte offsets / total
    int32_t grid;      // persistent CTAs (0: SMs x occupancy)
    int32_t codelet;   // compile-time specialised kernel id, -1 for the generic kernel
    int32_t ngroups;   // codelets: transform groups per CTA
    int32_t group_bytes;  // codelets: shared bytes per group (barriers, slots, work buffer)
    // codelets, even C2R: optional real weights multiplied into the input
    // bins as they are loaded (bin k of transform t times wload[t*wdist + k])
    const float* wload;
    int64_t wdist;
    // codelets: `in` is host memory mapped into the device's address space
    // (pinned host buffers): slots are filled by per-thread cp.async instead
    // of bulk copies
    int32_t host_in;
};

// Strided ("column") transforms, optionally one outer Stockham pass of a
// longer transform.  Column c (0 <= c < ncols) belongs to item c / cpi and
// has local index j = c % cpi; element r of it is read from
//   in  + item*in_dist  + (j / in_split)*in_hi  + (j % in_split)*in_lo  + r*in_stride
// and output bin k is written to
//   out + item*out_dist + (j / out_split)*out_hi + (j % out_split)*out_lo + k*out_stride
// (float2 units).  When ons > 1, input r is first multiplied by
// W_{ons*L}^{((j / tw_div) % ons) * r}, read as hi[m >> otw_shift] * lo[m & mask].
struct ColArgs {
    InnerPlan ip;
    const void* tw;
    const void* otw_hi;
    const void* otw_lo;
    const void* in;
    void* out;
    int64_t ncols;
    int64_t cpi;
    int64_t in_dist, in_split, in_hi, in_lo, in_stride;
    int64_t out_dist, out_split, out_hi, out_lo, out_stride;
    int64_t ons;
    int64_t tw_div;
    int32_t otw_shift;
    int32_t tfpc;      // columns per CTA
    int32_t tfp;       // shared-memory pitch in columns (>= tfpc)
    int32_t nbuf;      // shared buffers (1 or 2), each L*tfp float2
    int32_t pad_;
    int32_t conj_in;
    int32_t conj_out;
    int32_t staged_out;  // output of column c is out + c*L + k (contiguous blocks)
    float scale;
    // column-tile codelet (codelet >= 0): tfpc adjacent columns per tile, one
    // codelet transform group per column, column g held at g*wsize in shared
    // memory after the pass-table window [tw_lo, tw_lo + tw_cnt)
    int32_t codelet;
    int32_t tw_lo;
    int32_t tw_cnt;
    int32_t wsize;
    int32_t smem_bytes;
    int32_t pad2_;
};

// Stand-alone even/odd packing for R2C/C2R lengths beyond one CTA.
struct PackArgs {
    const void* in;
    void* out;
    const void* post_tw;  // W_N^k, k <= L/2
    int64_t ntf;
    int64_t in_dist, out_dist;  // float2 units
    int32_t L;                  // N/2
    int32_t c2r;                // 0: Z -> X (R2C post), 1: X -> conj(Z') (C2R pre)
    int32_t weight;
    float scale;
};

// Split-precision tensor-core sub-transforms of length L = R*R (R = 8 or
// 16): two DFT-matrix stages (R-point DFTs as [128 x 2R] x [2R x 2R] real
// GEMMs on tcgen05, operands split hi + lo, three products) with the W_L
// twiddle between them.  Sequence q = b*S + s, element n at
// in[b*in_dist + s*in_s + n*in_n]; output bin k at the same form with out_*,
// multiplied by W_N^{s*k} (N = S*L) when otw_hi is set.
enum TcIo : int32_t {
    TC_IO_GENERIC = 0,      // any strides (8-byte accesses)
    TC_IO_INTERLEAVED = 1,  // s stride 1: consecutive sequences side by side
    TC_IO_CONTIG = 2,       // n stride 1: each sequence contiguous
};
enum TcPrec : int32_t { TC_PREC_TF32X3 = 1, TC_PREC_BF16X3 = 2 };

struct TcArgs {
    const void* in;
    void* out;
    const void* bmat;    // DFT-matrix operand images (hi, then lo) in core-matrix layout
    const void* twl;     // W_L^j, j < L
    const void* otw_hi;  // W_N^{(e >> otw_shift) << otw_shift}; nullptr: no outer twiddle
    const void* otw_lo;  // W_N^{e & mask}
    int* err;
    int64_t nseq;
    int64_t S;
    int64_t in_dist, in_s, in_n;
    int64_t out_dist, out_s, out_n;
    int32_t R;
    int32_t prec;
    int32_t in_mode;
    int32_t out_mode;
    int32_t otw_shift;
    int32_t otw_hi_n;
    int32_t otw_lo_n;
    int32_t conj_in;
    int32_t conj_out;
    float scale;
};

// Ragged batches: many transforms of different lengths and kinds in one
// persistent launch.  A transform class (one kind and length) owns an
// on-chip plan; a work item is a group of same-class transforms done on chip
// (RAG_SINGLE), or one step of a long transform split as n' = L1*L2 (n' = n
// for C2C, n/2 for even R2C): RAG_P1 (a group of the L2 columns: length-L1
// transforms of x[j + L2*i] into the workspace), RAG_P2 (a group of the L1
// rows: twiddled length-L2 transforms from the workspace into the output,
// or into the second workspace half for R2C) and RAG_POST (even/odd
// post-process of a long R2C).  P2 items wait until all P1 items of their
// transform are done, POST items until all P2 items are; items are queued in
// that order, so every wait is on items already being processed.
enum RagType : int32_t { RAG_C2C = 0, RAG_R2C = 1 };
enum RagMode : int32_t { RAG_MODE_SINGLE = 0, RAG_MODE_LONG = 1 };
enum RagItemKind : int32_t { RAG_SINGLE = 0, RAG_P1 = 1, RAG_P2 = 2, RAG_POST = 3 };

struct RagClass {
    InnerPlan ip;      // single: the whole on-chip transform (length L); long: length L1
    InnerPlan ip2;     // long: length L2
    int32_t n;         // transform length
    int32_t type;      // RagType
    int32_t mode;      // RagMode
    int32_t L;         // complex length transformed (n for C2C and odd R2C, n/2 for even R2C)
    int32_t L1, L2;    // long: L = L1 * L2
    int32_t group;     // single: transforms per item; long: columns per P1 item
    int32_t group2;    // long: rows per P2 item
    int32_t pitch;     // single: shared-memory pitch of one transform (float2)
    int32_t otw_shift; // long: W_L^{k1*n2} = hi[e >> shift] * lo[e & mask]
    int64_t post_off;  // even R2C: W_n^k, k <= n/4 + 1 (float2 offset in the blob)
    int64_t hi_off, lo_off;
    // pass-table windows [tw_lo, tw_lo + tw_cnt) of ip and ip2, staged in
    // shared memory after the data buffers at float2 offset tw_smem
    int64_t tw_lo, tw2_lo;
    int32_t tw_cnt, tw2_cnt;
    int32_t tw_smem, tw2_smem;
};

struct RagXform {
    int64_t in_off;   // byte offsets from the exec's input / output pointers
    int64_t out_off;
    int64_t ws_off;   // long transforms: float2 offset of its workspace (2*L for R2C, L for C2C)
    int32_t cls;
    int32_t pad_;
};

struct RagItem {
    int32_t kind;   // RagItemKind
    int32_t cls;
    int32_t first;  // single: index into the order array; P1/P2: first column / row
    int32_t count;  // transforms / columns / rows in this item
    int32_t xform;  // P1/P2/POST: the transform
    int32_t need;   // P2/POST: completed items of the transform to wait for
};

struct RagArgs {
    const RagClass* cls;
    const RagXform* xf;
    const int32_t* order;  // single items: transform indices grouped by class
    const RagItem* items;
    int32_t nitems;
    int32_t smem_bytes;
    int32_t ctas;   // persistent CTAs to launch (gfft_ragged_ctas * SM count)
    int32_t need_bias;  // added to every dependency count (test hook; 0 normally)
    int* queue;     // queue[0]: next item; queue[1 + x]: completed items of transform x
    int* err;
    const void* tw;
    const void* in;
    void* out;
    void* ws;  // float2 workspace
    int32_t inverse;  // C2C transforms run backward (R2C transforms are always forward)
    float scale_c2c;  // applied to C2C outputs
    long long wait_cycles;  // bound of each dependency wait (SM clock cycles)
};

// Long C2C transforms on a thread-block cluster (csrc/cluster_fft.cu).  The
// length N = Q*P is split over the C CTAs of one cluster: CTA c loads the
// columns [c*P/C, (c+1)*P/C) of the Q x P row-major view of the input, runs
// the Q-point column transforms and the W_N^{p*k_q} twiddle, and stores each
// (Q/C) x (P/C) block into the shared memory of the CTA that owns those rows;
// CTA d then runs the P-point transforms of rows [d*Q/C, (d+1)*Q/C) and
// writes bins k_q + Q*k_p.  One HBM read and one HBM write per element.
// Transform t reads in + t*in_dist and writes out + t*out_dist (float2
// units); the clusters are persistent over transforms.
struct ClusterArgs {
    const void* in;
    void* out;
    const void* tw;     // twiddle blob
    int* err;           // device error word (bit 3: an exchange wait timed out)
    int64_t ntf;        // transforms
    int64_t in_dist, out_dist;
    int64_t twq_off;    // blob offset: column-phase second-pass table, W_Q^{k*r} at r*Q0 + k
    int64_t twp_off;    // blob offset: row-phase second-pass table, W_P^{k*r} at r*P0 + k
    int64_t outer_off;  // blob offset: W_N^e, e < N
    int64_t post_off;   // real modes: blob offset of W_{2N}^i, i <= N
    int32_t kid;        // configuration id (csrc/cluster_list.h)
    int32_t csize;      // CTAs per cluster (must match the configuration)
    int32_t conj_in;
    int32_t conj_out;
    float scale;
    int32_t smem_bytes;
    int32_t clusters;   // co-resident clusters (set when the plan is prepared on a device)
    int32_t length;     // complex transform length N = Q*P
    int32_t io_mode;    // IO_C2C; IO_R2C_EVEN / IO_C2R_EVEN: real length 2N with fused packing
    int32_t weight;     // WeightMode of the real modes
    int32_t pad_;
};

// Twiddle table segment: out[i] = W_M^{f(i)} (forward sign) with
//   kind 1: f(i) = (i * mult) mod M               (linear tables)
//   kind 2: f(i) = ((i / ns) * (i % ns)) mod M    (pass tables, [r][k] layout)
//   kind 3: the hi and lo operand images of the real-embedded R-point DFT
//           matrix (M = R, R_or_mult = TcPrec) for the tensor-core stages
struct TwSeg {
    int64_t offset;  // float2 offset in the table blob
    int64_t count;
    int64_t M;
    int64_t R_or_mult;
    int32_t kind;
    int32_t pad_;
};

}  // namespace gfft

// Launchers exported by the CUDA translation units (C linkage, plain types).
namespace gfft {

// Double-precision transforms: one radix-R Stockham pass, global memory to
// global memory.  Transform t (0 <= t < ntf) has element i at
//   base(t) + i*stride,  base(t) = (t / split)*hi + (t % split)*lo
// (double2 units; double units for a real input or output).  Butterfly j of
// the pass reads elements j + r*(n/R), multiplies them by W_{ns*R}^{(j%ns)*r}
// (read from the table W_n^m, m < n, at m = (j%ns)*r*n/(ns*R)), runs the
// R-point DFT and writes element (j/ns)*ns*R + j%ns + r*ns.
enum DIo : int32_t {
    DIO_C2C = 0,       // complex in, complex out
    DIO_REAL_IN = 1,   // first pass of a D2Z: real input, imaginary parts zero
    DIO_HERM_IN = 2,   // first pass of a Z2D: bins 0..n/2 of a Hermitian
                       // spectrum, expanded and conjugated (the backward
                       // transform as a forward one)
    DIO_HALF_OUT = 4,  // last pass of a D2Z: bins 0..n/2 only
    DIO_REAL_OUT = 8,  // last pass of a Z2D: real parts only
    // even N (n = 2L): not a pass but the real-data step around an L-point
    // transform; rows of L complex values (the real row viewed as complex)
    DIO_R2C_POST = 16,  // Z (L values) -> X (L + 1 bins), even/odd post-process
    DIO_C2R_PRE = 32,   // X (L + 1 bins) -> conj(Z') (L values), Hermitian pre-process
    DIO_PAIR_IN = 64,   // complex input read as two doubles (a real row viewed as
                        // complex: 8-byte alignment suffices)
    DIO_PAIR_OUT = 128, // complex output written as two doubles
};
struct DPassArgs {
    const void* in;
    void* out;
    const void* tw;  // double2 W_n^m, m < n
    int64_t ntf;
    int64_t in_split, in_hi, in_lo, in_stride;
    int64_t out_split, out_hi, out_lo, out_stride;
    int32_t n;
    int32_t radix;
    int32_t ns;
    int32_t io;        // DIo bits
    int32_t conj_in;   // conjugate on load (backward C2C)
    int32_t conj_out;  // conjugate on store
    int32_t t_fast;    // 1: consecutive threads take consecutive transforms (strided axes)
    int32_t pad_;
    double scale;
};

}  // namespace gfft

extern "C" {
int gfft_launch_dpass(const gfft::DPassArgs* a, void* stream);
// Fills table[m] = exp(-2 pi i m / n) in FP64 for m < n.
int gfft_gen_dtwiddles(void* table, long long n, void* stream);
int gfft_launch_row(const gfft::RowArgs* a, void* stream);
int gfft_launch_col(const gfft::ColArgs* a, void* stream);
int gfft_launch_pack(const gfft::PackArgs* a, void* stream);
int gfft_launch_tc(const gfft::TcArgs* a, void* stream);
int gfft_launch_ragged(const gfft::RagArgs* a, void* stream);
int gfft_launch_cluster(const gfft::ClusterArgs* a, void* stream);
// Cluster configuration for length n (csrc/cluster_list.h): returns its id
// (or -1) and fills the cluster size, the column/row lengths, their first
// radices, the threads per CTA and the dynamic shared memory per CTA.  want_c > 0 selects that cluster size.
int gfft_cluster_lookup(long long n, int want_c, int* csize, int* q, int* p, int* q0, int* p0, int* nt, int* smem_bytes);
// Sets the kernel attributes of configuration kid (io mode `mode`) on the current device and
// returns how many of its clusters are co-resident (negative CUDA error on
// failure).  Not stream-ordered: call outside stream capture.
int gfft_cluster_prepare(int kid, int mode);
// Prepares the ragged kernel for a shared-memory size (attributes) and
// returns its resident CTAs per SM (0 on error).  Not stream-ordered: call
// outside stream capture.
int gfft_ragged_ctas(int smem_bytes);
// float2 entries of the two DFT-matrix operand images for (R, prec).
long long gfft_tc_bmat_entries(int R, int prec);
int gfft_tc_gen_bmat(void* dst, int R, int prec, void* stream);
int gfft_gen_twiddles(void* table, const gfft::TwSeg* segs, int nseg, void* stream);
int gfft_kernel_max_threads(int rmax);
// Compile-time specialised row kernel for length L: returns its id (or -1)
// and fills its thread count per transform and radix sequence.
int gfft_codelet_lookup(int L, int* nthr, int* radices, int* nradix);
int gfft_codelet_lookup2(int L, int* nthr, int* radices, int* nradix, int* max_threads_per_cta);
// id of the k-th codelet_list.h entry of length L (-1 if none)
int gfft_codelet_find(int L, int variant);
// the compile-time spec of codelet `id`: length, threads per transform,
// radices, launch bound (threads per CTA, CTAs per SM); -1 if no such id
int gfft_codelet_info(int id, int* L, int* nthr, int* radices, int* nradix, int* max_threads_per_cta,
                      int* min_ctas_per_sm);
}
