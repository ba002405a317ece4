/*
 * CPU oracle for the Winograd 3x3 conv2d operator — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference project's own correctness
 * machinery so that tests, the smoke check and the CPU baseline of the
 * benchmark can check the CUDA operator.  Nothing in the operator library
 * links or calls this code; it is the checker, never the thing measured.
 *
 * What is restated (reference paths are relative to the reference project):
 *   - conv2dcpu, the direct-convolution verifier (include/verfiy.h:5-44):
 *     fp16 x fp16 products (exact), double accumulation in the loop order
 *     n, k, i, j, c, kh, kw, skip of out-of-bounds taps, one final rounding
 *     of the double sum to fp16.  Also returns the double sum itself: that
 *     is the FP64 oracle.
 *   - the benchmark's input generator (src/main.cpp:36-44): glibc rand()
 *     with its default seed, (rand()%255)/255.0 rounded to fp16, the input
 *     first, then the weights.
 *   - the algorithm selection of getkernelInfo (src/conv2d.cpp:76-114), in
 *     the reference's unsigned 32-bit arithmetic and with the tile
 *     constants it starts with (src/conv2d.cpp:3-8).
 *
 * Parity of this restatement is pinned against the reference's own
 * conv2dcpu compiled from the reference sources (oracle/Makefile builds
 * oracle/_ref/libref_verify.so) and against committed golden vectors made
 * by that build (tests/golden/).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---- IEEE binary16 <-> binary64, round to nearest even ----------------- */

double orc_half_to_double(uint16_t h)
{
    int sign = h >> 15;
    int exp = (h >> 10) & 0x1f;
    int mant = h & 0x3ff;
    double v;
    if (exp == 0)
        v = ldexp((double)mant, -24);
    else if (exp == 31)
        v = mant ? NAN : INFINITY;
    else
        v = ldexp((double)(mant + 1024), exp - 25);
    return sign ? -v : v;
}

/* Single rounding from binary64 straight to binary16 (no detour through
 * binary32), which is what a C++ cast of a double to _Float16 does. */
uint16_t orc_double_to_half(double x)
{
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    uint16_t sign = (uint16_t)((b >> 48) & 0x8000u);
    int exp = (int)((b >> 52) & 0x7ff);
    uint64_t mant = b & 0xFFFFFFFFFFFFFull;
    if (exp == 0x7ff)
        return (uint16_t)(sign | 0x7c00u | (mant ? 0x200u : 0u));
    if (exp == 0)
        return sign; /* binary64 subnormals are far below half's range */
    int e = exp - 1023;
    if (e > 15)
        return (uint16_t)(sign | 0x7c00u);
    uint64_t sig = mant | (1ull << 52);
    int shift;
    unsigned hexp;
    if (e >= -14) {
        shift = 42;
        hexp = (unsigned)(e + 15);
    } else {
        shift = 42 + (-14 - e);
        hexp = 0;
        if (shift > 63)
            return sign;
    }
    uint64_t keep = sig >> shift;
    uint64_t rem = sig & ((1ull << shift) - 1);
    uint64_t halfway = 1ull << (shift - 1);
    if (rem > halfway || (rem == halfway && (keep & 1)))
        keep++;
    if (hexp) {
        if (keep == (1ull << 11)) {
            keep >>= 1;
            hexp++;
        }
        if (hexp >= 31)
            return (uint16_t)(sign | 0x7c00u);
        return (uint16_t)(sign | (hexp << 10) | (unsigned)(keep & 0x3ff));
    }
    return (uint16_t)(sign | (unsigned)keep);
}

void orc_double_to_half_array(const double *x, uint16_t *out, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        out[i] = orc_double_to_half(x[i]);
}

void orc_half_to_double_array(const uint16_t *h, double *out, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        out[i] = orc_half_to_double(h[i]);
}

/* ---- glibc rand() (TYPE_3 additive feedback generator) ----------------- */
/* The reference benchmark never seeds rand(), so glibc starts from seed 1.
 * Restated from glibc's published srandom_r/random_r: a 31-word state
 * filled by the Park-Miller minimal standard generator, a separation of 3,
 * 310 discarded outputs, and each output the sum of two lagged words
 * shifted right by one. */
typedef struct {
    int32_t state[31];
    int f, r;
} orc_rng;

static int32_t orc_rng_next(orc_rng *g)
{
    uint32_t val = (uint32_t)g->state[g->f] + (uint32_t)g->state[g->r];
    g->state[g->f] = (int32_t)val;
    g->f = (g->f + 1) % 31;
    g->r = (g->r + 1) % 31;
    return (int32_t)(val >> 1);
}

static void orc_rng_seed(orc_rng *g, uint32_t seed)
{
    if (seed == 0)
        seed = 1;
    int32_t word = (int32_t)seed;
    g->state[0] = word;
    for (int i = 1; i < 31; ++i) {
        long hi = word / 127773;
        long lo = word % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0)
            w += 2147483647;
        word = (int32_t)w;
        g->state[i] = word;
    }
    g->f = 3;
    g->r = 0;
    for (int i = 0; i < 310; ++i)
        (void)orc_rng_next(g);
}

/* First `count` outputs of rand() after srand(seed). */
void orc_glibc_rand(uint32_t seed, int32_t *out, size_t count)
{
    orc_rng g;
    orc_rng_seed(&g, seed);
    for (size_t i = 0; i < count; ++i)
        out[i] = orc_rng_next(&g);
}

/* Input then weights, each element (rand()%255)/255.0 rounded to fp16,
 * exactly as src/main.cpp:36-44 fills them. */
void orc_fill_reference_style(uint16_t *in, size_t n_in, uint16_t *wt, size_t n_wt)
{
    orc_rng g;
    orc_rng_seed(&g, 1);
    for (size_t i = 0; i < n_in; ++i)
        in[i] = orc_double_to_half((orc_rng_next(&g) % 255) / 255.0);
    for (size_t i = 0; i < n_wt; ++i)
        wt[i] = orc_double_to_half((orc_rng_next(&g) % 255) / 255.0);
}

/* ---- direct convolution (include/verfiy.h:5-44) ------------------------ */

typedef struct {
    const uint16_t *in, *wt;
    uint16_t *out16;
    double *out64;
    long n, c, h, w, k, r, s, u, v, p, q, oh, ow;
    long plane_begin, plane_end; /* planes are (n, k) pairs */
} orc_conv_job;

static void orc_conv_planes(const orc_conv_job *J)
{
    const long c = J->c, h = J->h, w = J->w, k = J->k, r = J->r, s = J->s;
    const long oh = J->oh, ow = J->ow;
    double *wd = (double *)malloc(sizeof(double) * (size_t)(c * r * s));
    for (long pl = J->plane_begin; pl < J->plane_end; ++pl) {
        const long nn = pl / k, kk = pl % k;
        for (long t = 0; t < c * r * s; ++t)
            wd[t] = orc_half_to_double(J->wt[kk * r * s * c + t]);
        const uint16_t *img = J->in + nn * c * h * w;
        for (long i = 0; i < oh; ++i) {
            for (long j = 0; j < ow; ++j) {
                double sum = 0.0;
                const long posh = i * J->u - J->p;
                const long posw = j * J->v - J->q;
                for (long cc = 0; cc < c; ++cc) {
                    for (long kh = 0; kh < r; ++kh) {
                        for (long kw = 0; kw < s; ++kw) {
                            const long y = posh + kh, x = posw + kw;
                            if (x >= 0 && y >= 0 && x < w && y < h) {
                                /* both factors carry 11 significant bits, so
                                 * the product is exact in binary64 */
                                sum += orc_half_to_double(img[cc * h * w + y * w + x]) *
                                       wd[cc * r * s + kh * s + kw];
                            }
                        }
                    }
                }
                const long o = nn * k * oh * ow + kk * oh * ow + i * ow + j;
                if (J->out64)
                    J->out64[o] = sum;
                if (J->out16)
                    J->out16[o] = orc_double_to_half(sum);
            }
        }
    }
    free(wd);
}

static void *orc_conv_thread(void *arg)
{
    orc_conv_planes((const orc_conv_job *)arg);
    return NULL;
}

/* Returns 0 on success, -1 on a shape with no output.  out16 and/or out64
 * may be NULL.  nthreads <= 1 runs on the calling thread; otherwise the
 * (n, k) output planes are split across threads, which changes no result
 * because each output is one independent sum in a fixed order. */
int orc_conv2d_direct(const uint16_t *in, const uint16_t *wt, uint16_t *out16, double *out64,
                      int n, int c, int h, int w, int k, int r, int s, int u, int v, int p, int q,
                      int nthreads)
{
    orc_conv_job base;
    base.in = in;
    base.wt = wt;
    base.out16 = out16;
    base.out64 = out64;
    base.n = n; base.c = c; base.h = h; base.w = w; base.k = k;
    base.r = r; base.s = s; base.u = u; base.v = v; base.p = p; base.q = q;
    if (u <= 0 || v <= 0)
        return -1;
    base.oh = (h + 2L * p - r) / u + 1;
    base.ow = (w + 2L * q - s) / v + 1;
    if (base.oh <= 0 || base.ow <= 0)
        return -1;
    const long planes = (long)n * k;
    if (nthreads <= 1 || planes <= 1) {
        base.plane_begin = 0;
        base.plane_end = planes;
        orc_conv_planes(&base);
        return 0;
    }
    if (nthreads > planes)
        nthreads = (int)planes;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    orc_conv_job *jobs = (orc_conv_job *)malloc(sizeof(orc_conv_job) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = base;
        jobs[t].plane_begin = planes * t / nthreads;
        jobs[t].plane_end = planes * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, orc_conv_thread, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    return 0;
}

/* ---- algorithm selection (src/conv2d.cpp:76-114) ----------------------- */
/* 0 = F(4x3) non-fused, 1 = F(2x3) non-fused, 2 = F(2x3) fused: the order
 * of enum winograd_select (include/common.h:140-144).  Arithmetic is the
 * reference's unsigned 32-bit arithmetic with the tile constants of a
 * process's first call (input tile 6, output tile 4). */
int orc_select_reference(unsigned n, unsigned c, unsigned h, unsigned w, unsigned k,
                         unsigned r, unsigned s, unsigned u, unsigned v, unsigned p, unsigned q)
{
    unsigned outh = (h - r + 2 * p) / u + 1;
    unsigned outw = (w - s + 2 * q) / v + 1;
    /* getTileShape of {n, k, outh, outw} with TILE_OUT = 4 (common.h:85-93) */
    uint64_t tiles = (uint64_t)n * (((uint64_t)outh + 3) / 4) * (((uint64_t)outw + 3) / 4);
    unsigned image_size = n * c * h * w;
    unsigned filter_size = k * c * r * s;
    unsigned U_size = 6u * 6u * k * c;
    unsigned V_size = (unsigned)(6u * 6u * tiles * c);
    if (image_size >= 10u * filter_size)
        return 2;
    if (U_size > 4u * V_size)
        return 1;
    return 0;
}
