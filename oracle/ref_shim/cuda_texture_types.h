/* Stand-in for the CUDA texture-reference API, which CUDA 12 removed, so that
 * the reference extractor (DMC_CUDA/DMC_CUDA/src/dmc.cu) compiles unmodified
 * with CUDA 13 for sm_103a.  Test infrastructure only: it is found through
 * the include path of oracle/build_ref.py, ahead of the reference's own
 * `#include "cuda_texture_types.h"` (dmc.cu:14).
 *
 * The reference declares its lookup tables as file-scope
 *     texture<T, cudaTextureType1D, cudaReadModeElementType> name;
 * (dmc.cu:664-679), binds them to device buffers with
 *     cudaBindTexture(0, name, device_pointer, channel_desc)
 * (dmc.cu:732-778) and reads them with tex1Dfetch(name, i).  Here `texture`
 * expands to a __device__ variable holding the bound pointer and element
 * count; tex1Dfetch reads the element, or 0 outside the bound memory, which
 * is what a 1-D fetch from linear memory returns there; cudaBindTexture
 * writes the pointer and the element count of the rest of the allocation
 * (cuMemGetAddressRange, taken through the runtime's driver entry points). */
#ifndef DMCREF_TEXTURE_SHIM_H
#define DMCREF_TEXTURE_SHIM_H

/* everything the reference includes later, included before the macro below */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_runtime_api.h>
#include <device_launch_parameters.h>
#include <climits>
#include <cmath>
#include <cassert>
#include <functional>
#include <iomanip>
#include <iostream>
#include <memory>
#include <vector>

template <class T, int Dim, enum cudaTextureReadMode Mode>
struct dmcref_texture {
    const T *ptr;
    unsigned long long count;
};

template <class T, int Dim, enum cudaTextureReadMode Mode>
__device__ __forceinline__ T tex1Dfetch(const dmcref_texture<T, Dim, Mode> &t, int i)
{
    return (i >= 0 && (unsigned long long)i < t.count) ? t.ptr[i] : T(0);
}

/* bytes from p to the end of the device allocation that holds p; 0 if unknown */
static inline unsigned long long dmcref_bytes_after(const void *p)
{
    typedef CUresult (*RangeFn)(CUdeviceptr *, size_t *, CUdeviceptr);
    static RangeFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess)
            return 0;
        fn = (RangeFn)f;
    }
    CUdeviceptr base = 0;
    size_t size = 0;
    if (fn(&base, &size, (CUdeviceptr)p) != CUDA_SUCCESS) return 0;
    return (unsigned long long)(base + size - (CUdeviceptr)p);
}

template <class T, int Dim, enum cudaTextureReadMode Mode>
inline cudaError_t cudaBindTexture(size_t *offset, const dmcref_texture<T, Dim, Mode> &tex, const void *dev,
                                   const cudaChannelFormatDesc &, size_t size = UINT_MAX)
{
    if (offset) *offset = 0;
    unsigned long long bytes = dmcref_bytes_after(dev);
    if (bytes == 0) return cudaErrorInvalidValue;
    if ((unsigned long long)size < bytes) bytes = size;
    dmcref_texture<T, Dim, Mode> h;
    h.ptr = (const T *)dev;
    h.count = bytes / sizeof(T);
    return cudaMemcpyToSymbol(tex, &h, sizeof(h));
}

#define texture __device__ dmcref_texture

#endif
