// Winograd transform arithmetic for F(2x2,3x3) and F(4x4,3x3), in fp32.
//
// Element order e = row * ALPHA + col, tile order p = b*tilesPerImg +
// th*tilesW + tw, as in the reference (include/common.h:113-120;
// V[h*TILE_IN_W + w] in src/winograd_2x3_non_fused.cpp:371-374).
//
//  F2      F(2x3) with the reference's matrices:
//            B^T  src/winograd_2x3_non_fused.cpp:321-375
//            G    src/winograd_2x3_non_fused.cpp:260-300
//            A^T  src/winograd_2x3_non_fused.cpp:184-227
//  F4Ref   F(4x3) with the reference's interpolation points 0, +-1, +-2:
//            B^T  src/winograd_4x3_non_fused.cpp:41-146
//            G    src/winograd_4x3_non_fused.cpp:342-404
//            A^T  src/winograd_4x3_non_fused.cpp:427-525
//  F4      F(4x3) with points 0, +-1, 1/2, -2 (same tile sizes and layouts).
//          With fp16 operands its largest output error is 2.5-3x smaller than
//          F4Ref's, which keeps F(4x3) inside a 2e-2 relative bound; F4Ref
//          stays selectable for parity studies.
#pragma once
#include <cuda_runtime.h>

namespace wg {

// 1-D transforms on ALPHA-vectors with a stride, so the same code applies
// along columns and rows.  All constants are exact in fp32 except the
// thirds and fifteenths of F4's G, which is applied once per weight set.
struct F2 {
    static constexpr int M = 2, ALPHA = 4;
    template <class T>
    __device__ __forceinline__ static void bt(const T* d, int sd, T* o, int so) {
        const T d0 = d[0], d1 = d[sd], d2 = d[2 * sd], d3 = d[3 * sd];
        o[0] = d0 - d2;
        o[so] = d1 + d2;
        o[2 * so] = d2 - d1;
        o[3 * so] = d1 - d3;
    }
    template <class T>
    __device__ __forceinline__ static void g(const T* d, int sd, T* o, int so) {
        const T g0 = d[0], g1 = d[sd], g2 = d[2 * sd];
        o[0] = g0;
        o[so] = 0.5f * (g0 + g1 + g2);
        o[2 * so] = 0.5f * (g0 - g1 + g2);
        o[3 * so] = g2;
    }
    template <class T>
    __device__ __forceinline__ static void at(const T* m, int sm, T* o, int so) {
        const T m0 = m[0], m1 = m[sm], m2 = m[2 * sm], m3 = m[3 * sm];
        o[0] = m0 + m1 + m2;
        o[so] = m1 - m2 - m3;
    }
};

struct F4Ref {
    static constexpr int M = 4, ALPHA = 6;
    template <class T>
    __device__ __forceinline__ static void bt(const T* d, int sd, T* o, int so) {
        const T d0 = d[0], d1 = d[sd], d2 = d[2 * sd], d3 = d[3 * sd], d4 = d[4 * sd], d5 = d[5 * sd];
        o[0] = 4.f * d0 - 5.f * d2 + d4;
        o[so] = -4.f * (d1 + d2) + d3 + d4;
        o[2 * so] = 4.f * (d1 - d2) - d3 + d4;
        o[3 * so] = 2.f * (d3 - d1) - d2 + d4;
        o[4 * so] = 2.f * (d1 - d3) - d2 + d4;
        o[5 * so] = 4.f * d1 - 5.f * d3 + d5;
    }
    template <class T>
    __device__ __forceinline__ static void g(const T* d, int sd, T* o, int so) {
        const T g0 = d[0], g1 = d[sd], g2 = d[2 * sd];
        o[0] = g0 * (1.f / 4.f);
        o[so] = (g0 + g1 + g2) * (-1.f / 6.f);
        o[2 * so] = (g0 - g1 + g2) * (-1.f / 6.f);
        o[3 * so] = g0 * (1.f / 24.f) + g1 * (1.f / 12.f) + g2 * (1.f / 6.f);
        o[4 * so] = g0 * (1.f / 24.f) - g1 * (1.f / 12.f) + g2 * (1.f / 6.f);
        o[5 * so] = g2;
    }
    template <class T>
    __device__ __forceinline__ static void at(const T* m, int sm, T* o, int so) {
        const T m0 = m[0], m1 = m[sm], m2 = m[2 * sm], m3 = m[3 * sm], m4 = m[4 * sm], m5 = m[5 * sm];
        const T a = m1 + m2, b = m1 - m2, c = m3 + m4, d = m3 - m4;
        o[0] = m0 + a + c;
        o[so] = b + 2.f * d;
        o[2 * so] = a + 4.f * c;
        o[3 * so] = b + 8.f * d + m5;
    }
};

struct F4 {
    static constexpr int M = 4, ALPHA = 6;
    template <class T>
    __device__ __forceinline__ static void bt(const T* d, int sd, T* o, int so) {
        const T d0 = d[0], d1 = d[sd], d2 = d[2 * sd], d3 = d[3 * sd], d4 = d[4 * sd], d5 = d[5 * sd];
        o[0] = d0 + 1.5f * (d3 - d1) - 2.f * d2 + d4;
        o[so] = -d1 + 0.5f * d2 + 2.5f * d3 + d4;
        o[2 * so] = d1 - 2.5f * d2 + 0.5f * d3 + d4;
        o[3 * so] = 2.f * (d3 - d1) - d2 + d4;
        o[4 * so] = 0.5f * (d1 - d3) - d2 + d4;
        o[5 * so] = d1 + 1.5f * (d4 - d2) - 2.f * d3 + d5;
    }
    template <class T>
    __device__ __forceinline__ static void g(const T* d, int sd, T* o, int so) {
        const T g0 = d[0], g1 = d[sd], g2 = d[2 * sd];
        o[0] = g0;
        o[so] = (g0 + g1 + g2) * (1.f / 3.f);
        o[2 * so] = (g0 - g1 + g2) * (-1.f / 3.f);
        o[3 * so] = (16.f * g0 + 8.f * g1 + 4.f * g2) * (-1.f / 15.f);
        o[4 * so] = (g0 - 2.f * g1 + 4.f * g2) * (1.f / 15.f);
        o[5 * so] = g2;
    }
    template <class T>
    __device__ __forceinline__ static void at(const T* m, int sm, T* o, int so) {
        const T m0 = m[0], m1 = m[sm], m2 = m[2 * sm], m3 = m[3 * sm], m4 = m[4 * sm], m5 = m[5 * sm];
        const T a = m1 + m2, b = m1 - m2;
        o[0] = m0 + a + m3 + m4;
        o[so] = b + 0.5f * m3 - 2.f * m4;
        o[2 * so] = a + 0.25f * m3 + 4.f * m4;
        o[3 * so] = b + 0.125f * m3 - 8.f * m4 + m5;
    }
};

// 2-D transforms on row-major ALPHA x ALPHA (or 3x3) register arrays.
template <class TF>
__device__ __forceinline__ void input_tile_transform(const float (&d)[TF::ALPHA * TF::ALPHA],
                                                     float (&v)[TF::ALPHA * TF::ALPHA]) {
    constexpr int A = TF::ALPHA;
    float t[A * A];
#pragma unroll
    for (int j = 0; j < A; ++j) TF::bt(&d[j], A, &t[j], A);      // columns: B^T d
#pragma unroll
    for (int i = 0; i < A; ++i) TF::bt(&t[i * A], 1, &v[i * A], 1);  // rows: (B^T d) B
}

template <class TF>
__device__ __forceinline__ void filter_tile_transform(const float (&g)[9], float (&u)[TF::ALPHA * TF::ALPHA]) {
    constexpr int A = TF::ALPHA;
    float t[A * 3];
#pragma unroll
    for (int j = 0; j < 3; ++j) TF::g(&g[j], 3, &t[j], 3);       // G g
#pragma unroll
    for (int i = 0; i < A; ++i) TF::g(&t[i * 3], 1, &u[i * A], 1);  // (G g) G^T
}

template <class TF>
__device__ __forceinline__ void output_tile_transform(const float (&m)[TF::ALPHA * TF::ALPHA],
                                                      float (&y)[TF::M * TF::M]) {
    constexpr int A = TF::ALPHA, M = TF::M;
    float t[M * A];
#pragma unroll
    for (int j = 0; j < A; ++j) TF::at(&m[j], A, &t[j], A);      // A^T m
#pragma unroll
    for (int i = 0; i < M; ++i) TF::at(&t[i * A], 1, &y[i * M], 1);  // (A^T m) A
}

}  // namespace wg
