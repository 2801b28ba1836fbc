// Device side of the binary-block checkpoint format: the byte stream of
// saveBinaryBlock (io/serializerIO_3D.cpp:37-49) is a base64 text -- the
// size header and the cell records encoded separately, standard alphabet,
// '=' padding, no line breaks (io/base64.hh:35-115, io/serializerIO.cpp:64-86)
// -- and the records are built, encoded and decoded in device memory so that
// only the text crosses to the host.
#include <cuda_runtime.h>

#include <cstdint>

#include "launch.h"

namespace plbgpu {

namespace {

__device__ __forceinline__ char enc64(unsigned v) {
    return v < 26 ? (char)('A' + v) : v < 52 ? (char)('a' + v - 26) : v < 62 ? (char)('0' + v - 52)
                                                                     : (v == 62 ? '+' : '/');
}

// Value of a base64 character, or 64 for anything outside the alphabet.
__device__ __forceinline__ unsigned dec64(unsigned char c) {
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    return 64;
}

// Byte i of the stream head[0..headLen) ++ body[0..bodyLen).
__device__ __forceinline__ unsigned byteAt(const uint8_t* head, int headLen, const uint8_t* body, size_t i) {
    return i < (size_t)headLen ? head[i] : body[i - headLen];
}

// Quad t encodes stream bytes 3t .. 3t+2; the last quad of the stream may
// cover one or two bytes only and is then padded with '='.
__global__ void encodeKernel(const uint8_t* head, int headLen, const uint8_t* body, size_t bodyLen, size_t quads,
                             char* out) {
    const size_t total = (size_t)headLen + bodyLen;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < quads; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = 3 * t;
        const unsigned b0 = byteAt(head, headLen, body, i);
        const unsigned b1 = i + 1 < total ? byteAt(head, headLen, body, i + 1) : 0u;
        const unsigned b2 = i + 2 < total ? byteAt(head, headLen, body, i + 2) : 0u;
        char* o = out + 4 * t;
        o[0] = enc64(b0 >> 2);
        o[1] = enc64(((b0 & 0x03u) << 4) | (b1 >> 4));
        o[2] = i + 1 < total ? enc64(((b1 & 0x0fu) << 2) | (b2 >> 6)) : '=';
        o[3] = i + 2 < total ? enc64(b2 & 0x3fu) : '=';
    }
}

// Quads -> bytes; `bytes` is the number of bytes the quads hold (the last
// quad may be padded).  A character outside the alphabet (or a misplaced '=')
// sets *bad.
__global__ void decodeKernel(const char* in, size_t quads, size_t bytes, uint8_t* out, unsigned* bad) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < quads; t += (size_t)gridDim.x * blockDim.x) {
        const unsigned char* q = reinterpret_cast<const unsigned char*>(in) + 4 * t;
        const size_t i = 3 * t;
        const int keep = bytes - i >= 3 ? 3 : (int)(bytes - i);
        unsigned v[4];
        bool ok = true;
        for (int k = 0; k < 4; ++k) {
            const bool padded = k >= keep + 1;
            v[k] = padded ? (q[k] == '=' ? 0u : 64u) : dec64(q[k]);
            ok = ok && v[k] < 64u;
        }
        if (!ok) atomicOr(bad, 1u);
        const unsigned b0 = (v[0] << 2) | (v[1] >> 4);
        const unsigned b1 = ((v[1] & 0x0fu) << 4) | (v[2] >> 2);
        const unsigned b2 = ((v[2] & 0x03u) << 6) | v[3];
        out[i] = (uint8_t)b0;
        if (keep > 1) out[i + 1] = (uint8_t)b1;
        if (keep > 2) out[i + 2] = (uint8_t)b2;
    }
}

// out[c * outStride + outOff + k] = in[c * inStride + inOff + k], k < m.
__global__ void columnsKernel(const double* in, int inStride, int inOff, int m, double* out, int outStride,
                              int outOff, long long cells) {
    const long long total = cells * m;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long c = t / m;
        const int k = (int)(t - c * m);
        out[c * outStride + outOff + k] = in[c * inStride + inOff + k];
    }
}

unsigned gridFor(size_t work) {
    size_t b = (work + 255) / 256;
    return (unsigned)(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

}  // namespace

void launchBase64Encode(const uint8_t* head, int headLen, const uint8_t* body, size_t bodyLen, size_t quads,
                        char* out, cudaStream_t s) {
    encodeKernel<<<gridFor(quads), 256, 0, s>>>(head, headLen, body, bodyLen, quads, out);
}

void launchBase64Decode(const char* in, size_t quads, size_t bytes, uint8_t* out, unsigned* bad, cudaStream_t s) {
    decodeKernel<<<gridFor(quads), 256, 0, s>>>(in, quads, bytes, out, bad);
}

void launchColumns(const double* in, int inStride, int inOff, int m, double* out, int outStride, int outOff,
                   long long cells, cudaStream_t s) {
    columnsKernel<<<gridFor((size_t)cells * m), 256, 0, s>>>(in, inStride, inOff, m, out, outStride, outOff,
                                                             cells);
}

}  // namespace plbgpu
