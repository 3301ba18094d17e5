// The stage's image products (output_buffers, core/buffers.h:197-250), written from HBM.
//
//   k_rgbe         float RGB (or one plane as grey) -> Radiance RGBE bytes, per pixel: the largest
//                  component m gives the shared exponent e (m = f 2^e, f in [0.5, 1)) and each
//                  component c the mantissa byte floor(c f 256 / m), as stb_image_write encodes
//                  HDR files (the reference's Image::save). RGBE has no sign: a negative component
//                  is written as 0.
//   k_tonemap      float RGB -> 8-bit RGB through shared/image.h's curves (AgX with its default,
//                  golden and punchy looks, image.h:42-99; ACES, 29-40) and the byte conversion of
//                  Image::save_with_tonemapping (image.h:129-139), in the same single-precision
//                  operations (log2 and pow are CUDA's: a byte can differ by one where a value
//                  lands on a rounding boundary)
//   k_count_max /
//   k_count_fraction  normalized_sample_counts (core/buffers.h:183-195)
// The host side writes the bytes: a Radiance file (header and run-length-encoded scanlines) or
// a PNG (8-bit RGB, the image data in stored deflate blocks).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

__global__ void k_rgbe(Img3 src, int64_t np, uint8_t* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float c[3] = {float(src.at(i, 0)), float(src.at(i, 1)), float(src.at(i, 2))};
    const float m = fmaxf(c[0], fmaxf(c[1], c[2]));
    uint8_t b[4] = {0, 0, 0, 0};
    if (m >= 1e-32f) {
        int e = 0;
        const float scale = float(frexp(double(m), &e)) * 256.0f / m;
        for (int k = 0; k < 3; ++k) b[k] = uint8_t(fmaxf(c[k] * scale, 0.0f));
        b[3] = uint8_t(e + 128);
    }
    reinterpret_cast<uchar4*>(out)[i] = make_uchar4(b[0], b[1], b[2], b[3]);
}

// Row i of a 3x3 matrix times v, in Eigen's 3-vector dot order.
__device__ __forceinline__ float row_dot(float a, float b, float c, float x, float y, float z) {
    return dot3(a, b, c, x, y, z);
}

// Image::tone_map_Agx (shared/image.h:42-99)
__device__ void agx(const float in[3], int preset, float out[3]) {
    float col[3] = {row_dot(0.842479062253094f, 0.0423282422610123f, 0.0423756549057051f, in[0], in[1], in[2]),
                    row_dot(0.0784335999999992f, 0.878468636469772f, 0.0784336f, in[0], in[1], in[2]),
                    row_dot(0.0792237451477643f, 0.0791661274605434f, 0.879142973793104f, in[0], in[1], in[2])};
    const float min_ev = -12.47393f, max_ev = 4.026069f, ev_range = max_ev - min_ev;
    for (int k = 0; k < 3; ++k) {
        col[k] = fmaxs(col[k], 1e-8f);
        float enc = log2f(fmaxs(col[k], 1e-8f));
        enc = fclamps(enc, min_ev, max_ev);
        col[k] = (enc - min_ev) / ev_range;
    }
    float slope[3] = {1.0f, 1.0f, 1.0f}, power = 1.0f, saturation = 1.0f;
    if (preset == RPD_TONEMAP_AGX_GOLDEN) {
        slope[1] = 0.9f;
        slope[2] = 0.5f;
        power = 0.8f;
        saturation = 0.8f;
    } else if (preset == RPD_TONEMAP_AGX_PUNCHY) {
        power = 1.35f;
        saturation = 1.4f;
    }
    float val[3];
    for (int k = 0; k < 3; ++k) {
        const float x = col[k], x2 = x * x, x4 = x2 * x2, x6 = x4 * x2;
        const float x2x = x2 * x, x4x = x4 * x, x6x = x6 * x;
        const float poly = -17.86f * x6x + 78.01f * x6 - 126.7f * x4x + 92.06f * x4 - 28.72f * x2x + 4.361f * x2 -
                           0.1718f * x + 0.002857f;
        val[k] = powf(poly * slope[k], power);
    }
    const float luma = dot3(val[0], val[1], val[2], 0.2126f, 0.7152f, 0.0722f);
    for (int k = 0; k < 3; ++k) val[k] = luma + saturation * (val[k] - luma);
    const float res[3] = {
        row_dot(1.19687900512017f, -0.0528968517574562f, -0.0529716355144438f, val[0], val[1], val[2]),
        row_dot(-0.0980208811401368f, 1.15190312990417f, -0.0980434501171241f, val[0], val[1], val[2]),
        row_dot(-0.0990297440797205f, -0.0989611768448433f, 1.15107367264116f, val[0], val[1], val[2])};
    for (int k = 0; k < 3; ++k) out[k] = fmaxs(fmins(res[k], 1.0f), 0.0f);
}

// Image::tone_map_Aces (shared/image.h:29-40), with global.h's clamp
__device__ void aces(const float in[3], float out[3]) {
    const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
    for (int k = 0; k < 3; ++k) {
        const float c = 0.6f * in[k];
        const float v = (c * (A * c + B)) / (c * (C * c + D) + E);
        out[k] = fmaxs(fmins(v, 1.0f), 0.0f);  // clamp: cwiseMin(hi).cwiseMax(lo) (shared/global.h:41-43)
    }
}

__global__ void k_tonemap(Img3 src, int64_t np, int preset, uint8_t* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float in[3] = {float(src.at(i, 0)), float(src.at(i, 1)), float(src.at(i, 2))};
    float t[3];
    if (preset == RPD_TONEMAP_ACES) aces(in, t);
    else agx(in, preset, t);
    for (int k = 0; k < 3; ++k) out[3 * i + k] = uint8_t(255.0f * fmaxs(0.0f, fmins(1.0f, t[k])));
}

__global__ void k_count_max(const int32_t* __restrict__ counts, int64_t np, int* dmax) {
    int m = 1;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < np; i += int64_t(gridDim.x) * blockDim.x)
        m = max(m, counts[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(dmax, m);
}

__global__ void k_count_fraction(const int32_t* __restrict__ counts, int64_t np, const int* dmax, float* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float inv = 1.0f / float(*dmax);
    out[i] = float(max(0, counts[i])) * inv;
}

// ---- host: file formats --------------------------------------------------------------------

// CRC-32 (ISO 3309 polynomial 0xEDB88320), the PNG chunk checksum
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t k = 0; k < 256; ++k) {
            uint32_t c = k;
            for (int b = 0; b < 8; ++b) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[k] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
    static const CrcTable table;  // initialised once, thread-safely
    for (size_t i = 0; i < n; ++i) crc = table.t[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back(uint8_t(x >> 24));
    v.push_back(uint8_t(x >> 16));
    v.push_back(uint8_t(x >> 8));
    v.push_back(uint8_t(x));
}

void png_chunk(std::FILE* f, const char type[4], const std::vector<uint8_t>& data) {
    std::vector<uint8_t> buf;
    put_be32(buf, uint32_t(data.size()));
    buf.insert(buf.end(), type, type + 4);
    buf.insert(buf.end(), data.begin(), data.end());
    put_be32(buf, crc32_update(0xffffffffu, buf.data() + 4, buf.size() - 4) ^ 0xffffffffu);
    std::fwrite(buf.data(), 1, buf.size(), f);
}

bool write_png_file(const std::string& path, int w, int h, const uint8_t* rgb) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    std::fwrite(sig, 1, 8, f);
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, uint32_t(w));
    put_be32(ihdr, uint32_t(h));
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit RGB, deflate, adaptive filters, no interlace
    png_chunk(f, "IHDR", ihdr);
    // zlib stream of stored deflate blocks over the filtered rows (filter type 0 per row)
    const size_t row = size_t(w) * 3 + 1, raw = row * size_t(h);
    std::vector<uint8_t> z;
    z.reserve(raw + raw / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    uint32_t a = 1, b = 0;  // Adler-32
    std::vector<uint8_t> block;
    size_t done = 0;
    auto byte_at = [&](size_t k) -> uint8_t {
        const size_t y = k / row, x = k % row;
        return x == 0 ? 0 : rgb[y * size_t(w) * 3 + x - 1];
    };
    while (done < raw || raw == 0) {
        const size_t n = std::min<size_t>(65535, raw - done);
        z.push_back(done + n == raw ? 1 : 0);
        z.push_back(uint8_t(n));
        z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n));
        z.push_back(uint8_t(~n >> 8));
        for (size_t k = 0; k < n; ++k) {
            const uint8_t v = byte_at(done + k);
            z.push_back(v);
            a = (a + v) % 65521u;
            b = (b + a) % 65521u;
        }
        done += n;
        if (raw == 0) break;
    }
    put_be32(z, (b << 16) | a);
    png_chunk(f, "IDAT", z);
    png_chunk(f, "IEND", {});
    const bool ok = std::ferror(f) == 0;
    return std::fclose(f) == 0 && ok;
}

// One component of a Radiance scanline, run-length encoded: runs of 3 to 127 equal bytes as
// (128 + length, byte), everything else as literal groups of at most 128 (length, bytes...).
void rle_component(std::vector<uint8_t>& out, const uint8_t* v, int n) {
    int i = 0;
    while (i < n) {
        int run = 1;
        while (i + run < n && run < 127 && v[i + run] == v[i]) ++run;
        if (run >= 3) {
            out.push_back(uint8_t(128 + run));
            out.push_back(v[i]);
            i += run;
            continue;
        }
        // literals up to the next run of 3 (or 128 bytes)
        int j = i;
        while (j < n && j - i < 128) {
            if (j + 2 < n && v[j] == v[j + 1] && v[j] == v[j + 2]) break;
            ++j;
        }
        out.push_back(uint8_t(j - i));
        out.insert(out.end(), v + i, v + j);
        i = j;
    }
}

bool write_hdr_file(const std::string& path, int w, int h, const uint8_t* rgbe) {
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "#?RADIANCE\n# rpd-statmc-denoiser gb300\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", h, w);
    std::vector<uint8_t> line, comp(size_t(w) > 0 ? size_t(w) : 1);
    for (int y = 0; y < h; ++y) {
        const uint8_t* row = rgbe + size_t(y) * size_t(w) * 4;
        line.clear();
        if (w < 8 || w >= 32768) {  // outside the run-length form's range: flat RGBE
            line.assign(row, row + size_t(w) * 4);
        } else {
            line.insert(line.end(), {2, 2, uint8_t(w >> 8), uint8_t(w & 255)});
            for (int c = 0; c < 4; ++c) {
                for (int x = 0; x < w; ++x) comp[size_t(x)] = row[size_t(x) * 4 + c];
                rle_component(line, comp.data(), w);
            }
        }
        std::fwrite(line.data(), 1, line.size(), f);
    }
    const bool ok = std::ferror(f) == 0;
    return std::fclose(f) == 0 && ok;
}

}  // namespace

// Encode `src` (w x h) on `stream` into bytes and write the file: Radiance HDR (tonemap < 0) or
// tonemapped PNG. `dev` is scratch of at least 4 w h bytes, `host` page-locked of the same size.
int write_image(const Img3& src, int w, int h, int tonemap, const std::string& path, uint8_t* dev, uint8_t* host,
                cudaStream_t stream) {
    const int64_t np = int64_t(w) * h;
    if (tonemap < 0) k_rgbe<<<grid_for(np, 256), 256, 0, stream>>>(src, np, dev);
    else k_tonemap<<<grid_for(np, 256), 256, 0, stream>>>(src, np, tonemap, dev);
    RPD_CUDA(cudaGetLastError());
    const size_t bytes = size_t(np) * (tonemap < 0 ? 4 : 3);
    RPD_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, stream));
    RPD_CUDA(cudaStreamSynchronize(stream));
    const bool ok = tonemap < 0 ? write_hdr_file(path, w, h, host) : write_png_file(path, w, h, host);
    if (!ok) return fail(RPD_ERR_INVALID_ARGUMENT, "cannot write " + path);
    return RPD_OK;
}

cudaError_t launch_count_fraction(const int32_t* counts, int64_t np, int* dmax, float* out, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(dmax, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    k_count_max<<<304, 256, 0, stream>>>(counts, np, dmax);
    k_count_fraction<<<grid_for(np, 256), 256, 0, stream>>>(counts, np, dmax, out);
    return cudaGetLastError();
}

}  // namespace rpd
