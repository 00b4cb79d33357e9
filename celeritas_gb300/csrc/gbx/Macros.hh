// Function qualifiers of code shared by host and device.
#pragma once

#if defined(__CUDACC__)
#    define GBX_FUNCTION __host__ __device__
#    define GBX_FORCEINLINE __host__ __device__ __forceinline__
//! Kept out of line: rarely taken code that would otherwise be inlined at
//! every call site of a hot loop
#    define GBX_NOINLINE __host__ __device__ __noinline__ inline
#else
#    define GBX_FUNCTION
#    define GBX_FORCEINLINE inline
#    define GBX_NOINLINE inline
#endif
