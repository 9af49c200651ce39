// Project-written image codecs for scene import and frame output: zlib
// inflate (RFC 1950/1951), PNG decoding to RGBA8 (PNG 1.2: every colour type
// and bit depth, palette and tRNS transparency, Adam7 interlacing), and the
// CRC-32 / Adler-32 checksums PNG and zlib carry. The reference reads images
// through stb_image inside tinygltf (src/gltf_loader.cpp:532) and writes them
// through stb_image_write / OpenEXR; neither library is available here.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace optimg {

uint32_t crc32(const uint8_t *p, size_t n, uint32_t crc = 0);
uint32_t adler32(const uint8_t *p, size_t n, uint32_t a = 1);

// Raw DEFLATE stream -> bytes. Fails (returns false, message in err) on a
// malformed stream or when the output would exceed maxOut bytes.
bool inflate(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t maxOut, std::string &err);
// zlib stream (header, DEFLATE data, Adler-32 trailer) -> bytes.
bool zlibDecompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t maxOut, std::string &err);

struct Image {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> rgba;  // width * height * 4, rows top to bottom
};

bool isPng(const uint8_t *p, size_t n);
// Decodes a PNG to RGBA8 as stb_image does with four requested components:
// grey expands to (g, g, g), missing alpha is 255, 16-bit samples keep their
// high byte, low bit depths scale to 0..255, palette and tRNS apply.
bool decodePng(const uint8_t *p, size_t n, Image &img, std::string &err);

bool isJpeg(const uint8_t *p, size_t n);
// Decodes a baseline / extended-sequential (Huffman, 8-bit) JPEG to RGBA8
// (alpha 255): grey, YCbCr with any sampling factors (chroma upsampled by
// centred bilinear interpolation) or Adobe RGB; restart intervals and
// multi-scan frames. Progressive and arithmetic-coded files are errors.
bool decodeJpeg(const uint8_t *p, size_t n, Image &img, std::string &err);

// ---------------------------------------------------------------- encoders
// DEFLATE with dynamic Huffman codes (greedy LZ77 over a 32 KB window, hash
// chains; a block falls back to stored when that is smaller). `sync` ends
// the stream with an empty stored block instead of a final block, so that
// independently compressed pieces concatenate into one stream.
void deflate(const uint8_t *in, size_t n, std::vector<uint8_t> &out, bool sync);
// zlib stream of `n` bytes split into pieces compressed on up to `threads`
// host threads (piece boundaries on multiples of `grain` bytes).
void zlibCompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out, int threads, size_t grain);

// PNG (8-bit RGBA, colour type 6) of rows top to bottom; per-row filter
// chosen by the minimum sum of absolute residuals.
void encodePng(const uint8_t *rgba, uint32_t w, uint32_t h, size_t stride, std::vector<uint8_t> &out, int threads);
// Radiance RGBE (.hdr) from pre-converted RGBE pixels (4 bytes each), with
// run-length encoded scanlines for widths 8..32767.
void encodeHdr(const uint8_t *rgbe, uint32_t w, uint32_t h, std::vector<uint8_t> &out);
// OpenEXR scanline file, channels A, B, G, R as HALF; `rows` holds each
// scanline channel-planar (A[w], B[w], G[w], R[w] as 16-bit halves), the
// layout an EXR scanline stores. compression: 0 none, 3 ZIP (16 lines).
bool encodeExr(const uint16_t *rows, uint32_t w, uint32_t h, int compression, std::vector<uint8_t> &out, int threads);

}  // namespace optimg
