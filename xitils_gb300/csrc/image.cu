// Film -> 8-bit images and PNG files: the display / on-disk step after the film.
//
// Tonemap: RTCamp8/Main.cpp:669-682 maps a pixel's radiance v per channel to
// clamp((int)(pow(v * 0.3, 1 / 2.2) * 255), 0, 255); here the exposure (0.3)
// and gamma (2.2) are parameters and the film's sums are first scaled (1/spp).
// Error map: VisualizeError/Main.cpp:64-82 takes the squared difference of two
// images' luminance (rgbToLuminance, Vector.h:828-830), divides it by a maximum
// and colours it with the Jet colormap of tinycolormap (an un-vendored
// submodule, yuki-koyama/tinycolormap, no commit pinned): channel c is
// clamp(1.5 - 4 |t - m_c|, 0, 1) with m = 0.75, 0.5, 0.25 for r, g, b, t clamped
// to [0, 1]; the colour is stored as clamp((int)(c * 255), 0, 255).
// PNG: RGB8, rows top to bottom (film row 0 is the top of the image, since the
// film position flips y, RenderTarget.h:68-80), zlib stream of stored blocks.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/xgb.h"
#include "xgb_kernels.h"

namespace xgb {
bool filmPlane(xgb_film* f, void** d, int* w, int* h, int* fp64, int* device, cudaStream_t* ctxStream);
namespace {

__device__ __forceinline__ float filmChannel(const void* film, int fp64, size_t pix, int c) {
    return fp64 ? (float)((const double*)film)[4 * pix + c] : ((const float*)film)[4 * pix + c];
}

__device__ __forceinline__ unsigned char toByte(float v) {
    if (!(v == v)) return 0;  // NaN (a negative value under the power)
    float s = v * 255.0f;
    if (s >= 255.0f) return 255;
    if (s <= 0.0f) return 0;
    return (unsigned char)(int)s;
}

__global__ void k_tonemap(const void* film, int fp64, size_t n, float scale, float exposure, float invGamma,
                          unsigned char* rgb) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) {
            float v = filmChannel(film, fp64, i, c) * scale;
            rgb[3 * i + c] = toByte(powf(v * exposure, invGamma));
        }
}

// Film plane -> packed float RGB with `stride` floats per pixel (3 or 4), FP64
// films rounded to float: one linear device-to-host copy then moves the result
// (a strided 2D copy of 12-byte rows is slow on the copy engines).
__global__ void k_packFilm(const void* film, int fp64, size_t n, int stride, float* out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float r, g, b, w;
        if (fp64) {
            const double4 v = ((const double4*)film)[i];
            r = (float)v.x; g = (float)v.y; b = (float)v.z; w = (float)v.w;
        } else {
            const float4 v = __ldcs((const float4*)film + i);
            r = v.x; g = v.y; b = v.z; w = v.w;
        }
        if (stride == 4) {
            __stcs((float4*)out + i, make_float4(r, g, b, w));
        } else {
            out[3 * i] = r;
            out[3 * i + 1] = g;
            out[3 * i + 2] = b;
        }
    }
}

__device__ __forceinline__ float lum(float r, float g, float b) { return 0.298912f * r + 0.586611f * g + 0.114478f * b; }

__device__ __forceinline__ float jet(float t, float m) { return fminf(fmaxf(1.5f - 4.0f * fabsf(t - m), 0.0f), 1.0f); }

__global__ void k_errorMap(const void* a, int aFp64, float sa, const void* b, int bFp64, float sb, size_t n,
                           float invMax, unsigned char* rgb) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float la = lum(filmChannel(a, aFp64, i, 0) * sa, filmChannel(a, aFp64, i, 1) * sa, filmChannel(a, aFp64, i, 2) * sa);
        float lb = lum(filmChannel(b, bFp64, i, 0) * sb, filmChannel(b, bFp64, i, 1) * sb, filmChannel(b, bFp64, i, 2) * sb);
        float d = fabsf(la - lb);
        float t = fminf(fmaxf(d * d * invMax, 0.0f), 1.0f);
        rgb[3 * i] = toByte(jet(t, 0.75f));
        rgb[3 * i + 1] = toByte(jet(t, 0.5f));
        rgb[3 * i + 2] = toByte(jet(t, 0.25f));
    }
}

// ---- PNG -------------------------------------------------------------------
uint32_t crc32Table(int k) {
    uint32_t c = (uint32_t)k;
    for (int j = 0; j < 8; ++j) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

struct Crc {
    uint32_t table[256];
    Crc() { for (int k = 0; k < 256; ++k) table[k] = crc32Table(k); }
    uint32_t update(uint32_t c, const unsigned char* p, size_t n) const {
        for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
        return c;
    }
};

void put32(std::vector<unsigned char>& v, uint32_t x) {
    v.push_back((unsigned char)(x >> 24)); v.push_back((unsigned char)(x >> 16));
    v.push_back((unsigned char)(x >> 8)); v.push_back((unsigned char)x);
}

void chunk(std::vector<unsigned char>& out, const Crc& crc, const char* type, const std::vector<unsigned char>& data) {
    put32(out, (uint32_t)data.size());
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    uint32_t c = crc.update(0xFFFFFFFFu, out.data() + start, out.size() - start) ^ 0xFFFFFFFFu;
    put32(out, c);
}

}  // namespace

void launchPackFilm(const void* film, int fp64, size_t n, int strideFloats, float* out, int grid, cudaStream_t s) {
    k_packFilm<<<grid, 256, 0, s>>>(film, fp64, n, strideFloats, out);
}
}  // namespace xgb

using namespace xgb;

extern "C" {

xgb_status xgb_film_tonemap(xgb_film* film, float scale, float exposure, float gamma, unsigned char* rgb, void* stream) {
    void* d = nullptr;
    int w = 0, h = 0, fp64 = 0, device = 0;
    cudaStream_t st = nullptr;
    if (!film || !rgb || !(gamma > 0.0f) || !filmPlane(film, &d, &w, &h, &fp64, &device, &st)) return XGB_INVALID_ARG;
    cudaSetDevice(device);
    if (stream) st = (cudaStream_t)stream;
    size_t n = (size_t)w * h;
    unsigned char* dev = nullptr;
    if (cudaMallocAsync((void**)&dev, 3 * n, st) != cudaSuccess) return XGB_OOM;
    k_tonemap<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(d, fp64, n, scale, exposure, 1.0f / gamma, dev);
    cudaError_t e = cudaMemcpyAsync(rgb, dev, 3 * n, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dev, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? XGB_OK : XGB_CUDA_ERROR;
}

xgb_status xgb_film_error_map(xgb_film* a, float scale_a, xgb_film* b, float scale_b, float max_value,
                              unsigned char* rgb, void* stream) {
    void *da = nullptr, *db = nullptr;
    int wa = 0, ha = 0, fa = 0, wb = 0, hb = 0, fb = 0, deva = 0, devb = 0;
    cudaStream_t st = nullptr, stb = nullptr;
    if (!a || !b || !rgb || !(max_value > 0.0f) || !filmPlane(a, &da, &wa, &ha, &fa, &deva, &st) ||
        !filmPlane(b, &db, &wb, &hb, &fb, &devb, &stb) || wa != wb || ha != hb || deva != devb)
        return XGB_INVALID_ARG;
    cudaSetDevice(deva);
    if (stream) st = (cudaStream_t)stream;
    else if (stb != st) cudaStreamSynchronize(stb);
    size_t n = (size_t)wa * ha;
    unsigned char* dev = nullptr;
    if (cudaMallocAsync((void**)&dev, 3 * n, st) != cudaSuccess) return XGB_OOM;
    k_errorMap<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(da, fa, scale_a, db, fb, scale_b, n,
                                                                                  1.0f / max_value, dev);
    cudaError_t e = cudaMemcpyAsync(rgb, dev, 3 * n, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dev, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? XGB_OK : XGB_CUDA_ERROR;
}

xgb_status xgb_write_png(const char* path, int width, int height, const unsigned char* rgb) {
    if (!path || !rgb || width <= 0 || height <= 0) return XGB_INVALID_ARG;
    static const Crc crc;
    std::vector<unsigned char> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<unsigned char> ihdr;
    put32(ihdr, (uint32_t)width);
    put32(ihdr, (uint32_t)height);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, truecolour, deflate, no filter method, no interlace
    chunk(png, crc, "IHDR", ihdr);
    // image data: one filter byte (0) per row, in a zlib stream of stored deflate blocks
    const size_t row = (size_t)width * 3 + 1;
    std::vector<unsigned char> raw(row * height);
    for (int y = 0; y < height; ++y) {
        raw[y * row] = 0;
        std::memcpy(&raw[y * row + 1], rgb + (size_t)y * width * 3, (size_t)width * 3);
    }
    std::vector<unsigned char> z = {0x78, 0x01};
    uint32_t s1 = 1, s2 = 0;  // Adler-32
    for (unsigned char c : raw) { s1 = (s1 + c) % 65521u; s2 = (s2 + s1) % 65521u; }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        size_t len = std::min<size_t>(65535, raw.size() - off);
        bool last = off + len >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((unsigned char)(len & 0xFF)); z.push_back((unsigned char)(len >> 8));
        z.push_back((unsigned char)(~len & 0xFF)); z.push_back((unsigned char)((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (last) break;
    }
    put32(z, (s2 << 16) | s1);
    chunk(png, crc, "IDAT", z);
    chunk(png, crc, "IEND", {});
    FILE* f = std::fopen(path, "wb");
    if (!f) return XGB_INVALID_ARG;
    size_t wrote = std::fwrite(png.data(), 1, png.size(), f);
    std::fclose(f);
    return wrote == png.size() ? XGB_OK : XGB_INVALID_ARG;
}

}  // extern "C"
