// decode.cu — NIfTI voxel cast of load_nii (src/nii2mesh.c:160-175) on the
// device: img32[i] = (raw[i] * scl_slope) + scl_inter for the reference's
// four datatypes (uint8, int16, uint16, float32), a float multiply then a
// float add, each rounded (the reference's x86-64 build does not contract
// them).  Sending the raw voxels and casting here cuts the host-to-device
// bytes of an 8-bit volume to a quarter.
//
// Integer voxels become floats by bit assembly (exact for |v| < 2^23): this
// part issues I2F on the pipe it shares with FP64.
#include "n2m_internal.cuh"

namespace {
__device__ __forceinline__ float u2f_small(unsigned v) { return __int_as_float(0x4B000000 | (int)v) - 8388608.f; }

template <class T>
__device__ __forceinline__ float as_float(T v);
template <>
__device__ __forceinline__ float as_float<unsigned char>(unsigned char v) { return u2f_small(v); }
template <>
__device__ __forceinline__ float as_float<unsigned short>(unsigned short v) { return u2f_small(v); }
template <>
__device__ __forceinline__ float as_float<short>(short v) {
    return __fsub_rn(u2f_small((unsigned)((int)v + 32768)), 32768.f);
}
template <>
__device__ __forceinline__ float as_float<float>(float v) { return v; }

template <class T>
__global__ void __launch_bounds__(256) k_cast(const T *__restrict__ raw, float *__restrict__ out, long long n,
                                              float slope, float inter) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __fadd_rn(__fmul_rn(as_float<T>(raw[i]), slope), inter);
}
}  // namespace

int nifti_bytes_per_voxel(int datatype) {
    switch (datatype) {
    case N2M_DT_UINT8: return 1;
    case N2M_DT_INT16: case N2M_DT_UINT16: return 2;
    case N2M_DT_FLOAT32: return 4;
    default: return 0;
    }
}

n2m_status launch_cast(const void *d_raw, int datatype, float slope, float inter, long long n, float *d_out,
                       cudaStream_t s) {
    if (slope == 0.0f) slope = 1.0f;   // src/nii2mesh.c:122
    if (n <= 0) return N2M_OK;
    long long b = (n + 255) / 256;
    const unsigned blocks = (unsigned)(b < 152 * 16 ? b : 152 * 16);
    switch (datatype) {
    case N2M_DT_UINT8: k_cast<unsigned char><<<blocks, 256, 0, s>>>((const unsigned char *)d_raw, d_out, n, slope, inter); break;
    case N2M_DT_INT16: k_cast<short><<<blocks, 256, 0, s>>>((const short *)d_raw, d_out, n, slope, inter); break;
    case N2M_DT_UINT16: k_cast<unsigned short><<<blocks, 256, 0, s>>>((const unsigned short *)d_raw, d_out, n, slope, inter); break;
    case N2M_DT_FLOAT32: k_cast<float><<<blocks, 256, 0, s>>>((const float *)d_raw, d_out, n, slope, inter); break;
    default:
        n2m_set_error("unsupported NIfTI datatype %d (uint8 2, int16 4, float32 16, uint16 512)", datatype);
        return N2M_ERR_BAD_ARGS;
    }
    N2M_COUNT();
    CKL();
    return N2M_OK;
}
