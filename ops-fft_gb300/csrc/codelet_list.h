// codelet_list.h - the compile-time specialised row kernels that are built.
// X(id, MAXT, MINB, L, NTHR, radices...): launch bound of MAXT threads per CTA
// with MINB CTAs per SM (register cap 65536 / (MAXT * MINB)).  The first
// entry of a length is its fastest spill-free build: for 512-4096 points
// the higher register cap (the 80-register builds of 1024-4096 spill and
// ran up to 1.2x slower; the spill-free 80-register 512-point build is 3-6 %
// faster alone but made the R2C/C2R round trip over N=3000 and N=1024, whose
// two chains run concurrently, 6 % slower); for 1500 points the lower one
// (96 registers, 4 CTAs per SM: R2C N=3000 batch 4096 6 % faster than 108
// registers at 3 CTAs per SM, the round trip 5 % faster); for 128/256
// points the radix order that keeps all 32 lanes of the transform's warp
// busy (8*8*4: 1.17x, 4*4*8: 1.11x over 16*16 and 8*16); the planner
// picks the first entry whose length matches exactly, or the k-th one with
// OPS_FFT_CODELET_VARIANT=k (entries after the first for a length are
// variants: other register caps or radix orders; a column pass takes the
// entry of its length that holds 8 to 16 columns with the most threads
// resident per SM, then the most columns: entries 23-26 exist for that, the
// 512- and 1024-point column passes of 2D and 3D transforms, measured
// 15-34 % faster than the column kernel on 512^3, 64 x 1024^2, 8 x 1024^2
// and 64 x 512^2; entry 25's 16 columns of 512 points (32 threads each)
// another 12 % on 512^3, and entry 26's 8 columns at 3 CTAs per SM (80
// registers) another 10 % (512^3 2048 -> 1834 us, 64 x 512^2 169 -> 143 us;
// 2 CTAs per SM 1906 us, 4 CTAs per SM with spills 1845 us); 16-column
// builds for 256 and 1024 points, and 8 columns of 1024 points at 2 CTAs
// per SM (32 threads per column, 128 registers: 8 x 1024^2 83 -> 90 us; 64
// threads per column, 64 registers with a 48-byte spill: 85 -> 93 us,
// 64 x 1024^2 563 -> 623 us), were slower).  Each entry is
// instantiated in its own translation unit (codelet_<id>.cu) so the build
// runs in parallel.
#pragma once
#define GFFT_CODELETS(X)                       \
    X(0, 160, 4, 1500, 160, 15, 10, 10)        \
    X(1, 256, 2, 512, 64, 8, 8, 8)             \
    X(2, 256, 2, 4096, 256, 16, 16, 16)        \
    X(3, 256, 2, 2048, 128, 16, 16, 8)         \
    X(4, 256, 2, 1024, 64, 16, 16, 4)          \
    X(5, 256, 2, 256, 32, 8, 8, 4)             \
    X(6, 256, 2, 128, 32, 4, 4, 8)             \
    X(7, 512, 1, 8192, 512, 16, 16, 16, 2)     \
    X(8, 160, 6, 1500, 160, 15, 10, 10)        \
    X(9, 128, 8, 512, 64, 8, 8, 8)             \
    X(10, 1024, 1, 2048, 128, 16, 16, 8)       \
    X(11, 384, 2, 4096, 256, 16, 16, 16)       \
    X(12, 384, 2, 2048, 128, 16, 16, 8)        \
    X(13, 384, 2, 1024, 64, 16, 16, 4)         \
    X(14, 384, 2, 1500, 160, 15, 10, 10)       \
    X(15, 384, 2, 512, 64, 8, 8, 8)            \
    X(16, 384, 2, 256, 32, 16, 16)             \
    X(17, 384, 2, 128, 32, 8, 16)              \
    X(18, 256, 1, 1500, 32, 15, 10, 10)        \
    X(19, 256, 1, 1500, 32, 10, 10, 15)        \
    X(20, 256, 1, 1500, 64, 15, 10, 10)        \
    X(21, 160, 3, 1500, 160, 15, 10, 10)       \
    X(22, 256, 3, 512, 64, 8, 8, 8)            \
    X(23, 512, 1, 512, 64, 8, 8, 8)            \
    X(24, 512, 1, 1024, 64, 16, 16, 4)         \
    X(25, 512, 1, 512, 32, 8, 8, 8)        \
    X(26, 256, 3, 512, 32, 8, 8, 8)
#define GFFT_NUM_CODELETS 27
