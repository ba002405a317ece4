// C++-linkage entry points with the reference's mangled names
// (include/conv2d.h:39-40 declares getParamsize and getkernelInfo without
// extern "C").  A program compiled against the reference header links to
// these; they forward to the C-linkage implementation.  This translation
// unit deliberately does not include the library's own header, whose C
// declarations of the same names would conflict.
typedef struct
{
    void* in;
    void* weight;
    void* out;
    unsigned int n, c, h, w, k, r, s, u, v, p, q;
} problem_t;

typedef struct
{
    unsigned int blockx, blocky, blockz, threadx, thready, threadz, dynmicLdsSize;
    void* kernelPtr;
} kernelInfo_t;

extern "C" int wg_getParamsize(problem_t* problem, int* paramSize);
extern "C" int wg_getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param);

int getParamsize(problem_t* problem, int* paramSize) { return wg_getParamsize(problem, paramSize); }

int getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param)
{
    return wg_getkernelInfo(problem, kernelInfo, param);
}
