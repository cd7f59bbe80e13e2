/*
 * CUDA emulation prelude for running the reference's kernel source on the host.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is force-included ahead of the
 * unmodified reference translation unit (src/pCT_Reconstruction_Data_Segments.cu)
 * when oracle/build_ref.py compiles it with g++ into oracle/_ref/.  Nothing in
 * the product links against it.
 *
 * What it provides:
 *   - the CUDA qualifiers as no-ops, so __global__/__device__ functions become
 *     ordinary host functions;
 *   - threadIdx/blockIdx/blockDim/gridDim as globals that the harness sets while
 *     it walks a launch grid sequentially (one emulated thread at a time);
 *   - atomicAdd as a plain read-modify-write in the destination type (the value
 *     is converted to the destination type first, as CUDA's typed overloads do),
 *     which makes every float sum run in thread order;
 *   - the host memory API (cudaMalloc/cudaMemcpy/cudaFree ...) over malloc;
 *   - the global math overload set that nvcc 13 exposes (verified with
 *     static_asserts under nvcc): atan2(float,float)->float, abs(float)->float,
 *     abs(double)->double, pow(float,float)->float, pow(float,int)->double,
 *     plus CUDA's integer/double max/min;
 *   - correctly rounded binary32 atan2/sinf/cosf (the binary64 libm result
 *     rounded once).  The reference's results depend on these float functions
 *     bit for bit, and neither of its own builds has a canonical version
 *     (glibc 2.39 atan2f misrounds about one input in six; CUDA's atan2f is
 *     documented to 2 ulp), so the harness pins them to the exact value, the
 *     same definition the product and the oracle use;
 *   - correctly rounded binary64 sin/cos (the binary128 libquadmath value
 *     rounded once) for the same reason: glibc 2.39's sin and cos misround a
 *     few of the per-angle arguments the reference tabulates (gantry rotation,
 *     bin angles, backprojection), CUDA's are documented to 2 ulp, and the
 *     product and the oracle build those tables correctly rounded;
 *   - the two shims the reference needs under a modern compiler:
 *     `syncthreads` (undefined in CUDA) and `std::ifstream == NULL`.
 */
#ifndef PCT_REF_PRELUDE_H
#define PCT_REF_PRELUDE_H

#include <cmath>
#include <quadmath.h>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <fstream>
#include <ios>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

inline void __syncthreads() {}
#define syncthreads __syncthreads

template <class T, class U> inline T atomicAdd(T* address, U value) {
    T old = *address;
    *address = static_cast<T>(old + static_cast<T>(value));
    return old;
}

typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice };
typedef void* cudaEvent_t;
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = std::calloc(n ? n : 1, 1); return *p ? 0 : 2; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memmove(d, s, n); return 0; }
inline cudaError_t cudaFree(void* p) { std::free(p); return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline const char* cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaSetDevice(int) { return 0; }
inline cudaError_t cudaEventCreate(cudaEvent_t*) { return 0; }
inline cudaError_t cudaEventRecord(cudaEvent_t, int = 0) { return 0; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return 0; }
inline cudaError_t cudaEventElapsedTime(float* t, cudaEvent_t, cudaEvent_t) { *t = 0.f; return 0; }
inline cudaError_t cudaProfilerStart() { return 0; }
inline cudaError_t cudaProfilerStop() { return 0; }

/* Global math overloads matching nvcc's (see header comment). */
inline float atan2(float y, float x) { return (float)::atan2((double)y, (double)x); }
inline float pct_ref_sinf(float x) { return (float)::sin((double)x); }
inline float pct_ref_cosf(float x) { return (float)::cos((double)x); }
#define sinf pct_ref_sinf
#define cosf pct_ref_cosf
using std::abs;
using std::pow;
using std::sqrt;
using std::sin;
using std::cos;
using std::tan;
using std::log;
using std::exp;
using std::fabs;
using std::floor;
using std::ceil;
/* sin and cos: binary64 correctly rounded; the float overloads as sinf/cosf.
 * The reference takes sin and cos of the same angle at every MLP sample
 * (.cu:5465) and of each projection angle for every voxel it backprojects
 * (.cu:3180), so each thread remembers 4096 arguments of each (a
 * direct-mapped table on a hash of the argument's bits): binary128 is slow. */
enum { PCT_REF_MEMO = 4096 };
struct pct_ref_memo {
    unsigned long long key[PCT_REF_MEMO];
    double val[PCT_REF_MEMO];
    bool used[PCT_REF_MEMO];
};
inline double pct_ref_memo_get(pct_ref_memo& m, double x, __float128 (*f)(__float128)) {
    unsigned long long k;
    std::memcpy(&k, &x, sizeof k);
    const unsigned long long h = k * 0x9E3779B97F4A7C15ull;
    const int slot = (int)(h >> 52); /* 12 bits */
    if (m.used[slot] && m.key[slot] == k) return m.val[slot];
    const double v = (double)f((__float128)x);
    m.key[slot] = k;
    m.val[slot] = v;
    m.used[slot] = true;
    return v;
}
inline double pct_ref_sin(double x) {
    static thread_local pct_ref_memo m = {};
    return pct_ref_memo_get(m, x, sinq);
}
inline double pct_ref_cos(double x) {
    static thread_local pct_ref_memo m = {};
    return pct_ref_memo_get(m, x, cosq);
}
inline float pct_ref_sin(float x) { return pct_ref_sinf(x); }
inline float pct_ref_cos(float x) { return pct_ref_cosf(x); }
inline double pct_ref_sin(int x) { return pct_ref_sin((double)x); }
inline double pct_ref_cos(int x) { return pct_ref_cos((double)x); }
#define sin pct_ref_sin
#define cos pct_ref_cos
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, int b) { return max(a, (unsigned int)b); }
inline unsigned int max(int a, unsigned int b) { return max((unsigned int)a, b); }
inline unsigned int min(unsigned int a, int b) { return min(a, (unsigned int)b); }
inline unsigned int min(int a, unsigned int b) { return min((unsigned int)a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }

/* `std::ifstream == NULL` (reference .cu:1109,1154,1815,1980). */
inline bool operator==(const std::basic_ios<char>& s, long) { return !s; }

#endif
