// Test infrastructure only: exposes the reference project's own CPU verifier
// conv2dcpu (include/verfiy.h:5-44), compiled unmodified from the reference
// sources, behind a C symbol so the oracle's restatement can be pinned to it.
// Built by oracle/Makefile into oracle/_ref/; never linked into the operator.
#include <stdint.h>
#include <stdlib.h>
#include "verfiy.h"

extern "C" void ref_conv2dcpu(uint16_t *pin, uint16_t *pwei, uint16_t *pout, int n, int c, int h,
                              int w, int k, int r, int s, int u, int v, int p, int q)
{
    conv2dcpu(reinterpret_cast<_Float16 *>(pin), reinterpret_cast<_Float16 *>(pwei),
              reinterpret_cast<_Float16 *>(pout), n, c, h, w, k, r, s, u, v, p, q);
}

// The benchmark's input fill (src/main.cpp:36-44) run through the host
// compiler's own rand() and double -> _Float16 conversion.
extern "C" void ref_fill_reference_style(uint16_t *in, long n_in, uint16_t *wt, long n_wt)
{
    srand(1);
    _Float16 *pi = reinterpret_cast<_Float16 *>(in);
    _Float16 *pw = reinterpret_cast<_Float16 *>(wt);
    for (long i = 0; i < n_in; i++)
        pi[i] = (rand() % 255) / 255.0;
    for (long i = 0; i < n_wt; i++)
        pw[i] = (rand() % 255) / 255.0;
}
