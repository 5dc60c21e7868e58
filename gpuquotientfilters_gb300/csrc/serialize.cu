// Filter images: checkpoint / restore of SQF tables and RSQF blocks.
//
// Layout (little-endian), 64-byte header then the payload:
//   0  char[8]  magic    "GQFSQF01" | "GQFRSQF1"
//   8  u32      version  1
//  12  u32      q
//  16  u32      r        (SQF remainder bits; 5 for the RSQF)
//  20  u32      unit     bytes per slot (SQF) | bytes per block (RSQF, 57)
//  24  u64      payload  bytes that follow the header
//  32  u64      checksum FNV-1a 64 over the payload, 8-byte words
//  40  u8[24]   zero
// The payload is the device table as the reference lays it out (SQF
// quotientFilter.cu:151-170, RSQF RSQF.cuh:24-30), so an image restores bit
// for bit.  The RSQF guard block is all zero by construction and not stored.
#include <cstdio>
#include <cstring>
#include <vector>

#include "host_common.cuh"

namespace gqf {

static const char SQF_MAGIC[8] = {'G', 'Q', 'F', 'S', 'Q', 'F', '0', '1'};
static const char RSQF_MAGIC[8] = {'G', 'Q', 'F', 'R', 'S', 'Q', 'F', '1'};
constexpr uint32_t IMAGE_VERSION = 1;
constexpr uint32_t RSQF_BB = GQF_RSQF_BLOCK_BYTES;  // packed block (RSQF.cuh:24-30)
constexpr uint32_t RSQF_R = GQF_RSQF_RBITS;

struct ImageHeader {
    char magic[8];
    uint32_t version, q, r, unit;
    uint64_t payload, checksum;
    uint8_t zero[24];
};
static_assert(sizeof(ImageHeader) == GQF_IMAGE_HEADER_BYTES, "image header is 64 bytes");

// FNV-1a over little-endian 64-bit words (the tail zero-padded), a fast
// host checksum that catches truncation and bit damage.
static uint64_t image_checksum(const uint8_t *p, size_t n)
{
    uint64_t h = 1469598103934665603ull;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        memcpy(&w, p + i, 8);
        h = (h ^ w) * 1099511628211ull;
    }
    if (i < n) {
        uint64_t w = 0;
        memcpy(&w, p + i, n - i);
        h = (h ^ w) * 1099511628211ull;
    }
    return h;
}

static int save_image(const char *magic, uint32_t q, uint32_t r, uint32_t unit, const void *dev, size_t payload,
                      void *buf, size_t cap, cudaStream_t s)
{
    if (!buf || cap < sizeof(ImageHeader) + payload) return GQF_ERR_ARG;
    uint8_t *out = static_cast<uint8_t *>(buf);
    GQF_CK(cudaMemcpyAsync(out + sizeof(ImageHeader), dev, payload, cudaMemcpyDeviceToHost, s));
    GQF_CK(cudaStreamSynchronize(s));
    ImageHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, magic, 8);
    h.version = IMAGE_VERSION;
    h.q = q;
    h.r = r;
    h.unit = unit;
    h.payload = payload;
    h.checksum = image_checksum(out + sizeof(ImageHeader), payload);
    memcpy(out, &h, sizeof h);
    return GQF_OK;
}

static int parse_image(const char *magic, const void *buf, size_t len, ImageHeader &h)
{
    if (!buf || len < sizeof(ImageHeader)) return GQF_ERR_FORMAT;
    memcpy(&h, buf, sizeof h);
    if (memcmp(h.magic, magic, 8) != 0 || h.version != IMAGE_VERSION) return GQF_ERR_FORMAT;
    for (uint8_t z : h.zero)
        if (z) return GQF_ERR_FORMAT;
    if (len != sizeof(ImageHeader) + h.payload) return GQF_ERR_FORMAT;
    if (image_checksum(static_cast<const uint8_t *>(buf) + sizeof(ImageHeader), h.payload) != h.checksum)
        return GQF_ERR_FORMAT;
    return GQF_OK;
}

static int read_file(const char *path, std::vector<uint8_t> &v)
{
    if (!path) return GQF_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return GQF_ERR_IO;
    int st = GQF_OK;
    if (fseek(f, 0, SEEK_END) != 0) st = GQF_ERR_IO;
    long n = st ? -1 : ftell(f);
    if (n < 0 || fseek(f, 0, SEEK_SET) != 0) st = GQF_ERR_IO;
    if (!st) {
        v.resize((size_t)n);
        if (n > 0 && fread(v.data(), 1, (size_t)n, f) != (size_t)n) st = GQF_ERR_IO;
    }
    fclose(f);
    return st;
}

static int write_file(const char *path, const std::vector<uint8_t> &v)
{
    if (!path) return GQF_ERR_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return GQF_ERR_IO;
    const bool ok = fwrite(v.data(), 1, v.size(), f) == v.size();
    return (fclose(f) == 0 && ok) ? GQF_OK : GQF_ERR_IO;
}

}  // namespace gqf

using namespace gqf;

extern "C" {

size_t gqf_sqf_image_bytes(const gqf_sqf *qf)
{
    return qf ? sizeof(ImageHeader) + gqf_sqf_table_bytes(qf->qbits, qf->rbits) : 0;
}

size_t gqf_rsqf_image_bytes(const gqf_rsqf *cqf)
{
    return cqf ? sizeof(ImageHeader) + (size_t)cqf->numBlocks * RSQF_BB : 0;
}

int gqf_sqf_save(const gqf_sqf *qf, void *buf, size_t cap, void *stream)
{
    if (!qf || !qf->table) return GQF_ERR_ARG;
    return save_image(SQF_MAGIC, qf->qbits, qf->rbits, qf->bytesPerElement, qf->table,
                      gqf_sqf_table_bytes(qf->qbits, qf->rbits), buf, cap, static_cast<cudaStream_t>(stream));
}

int gqf_rsqf_save(const gqf_rsqf *cqf, void *buf, size_t cap, void *stream)
{
    if (!cqf || !cqf->blocks || cqf->numBlocks != gqf_rsqf_num_blocks(cqf->qbits)) return GQF_ERR_ARG;
    return save_image(RSQF_MAGIC, cqf->qbits, RSQF_R, RSQF_BB, cqf->blocks, (size_t)cqf->numBlocks * RSQF_BB, buf,
                      cap, static_cast<cudaStream_t>(stream));
}

int gqf_sqf_load(gqf_sqf *qf, const void *buf, size_t len)
{
    if (!qf) return GQF_ERR_ARG;
    ImageHeader h;
    int st = parse_image(SQF_MAGIC, buf, len, h);
    if (st) return st;
    gqf_sqf tmp;
    st = gqf_sqf_init(&tmp, h.q, h.r);
    if (st) return st == GQF_ERR_ARG ? GQF_ERR_FORMAT : st;
    if (h.payload != gqf_sqf_table_bytes(h.q, h.r) || h.unit != tmp.bytesPerElement) {
        gqf_sqf_free(&tmp);
        return GQF_ERR_FORMAT;
    }
    cudaError_t e = cudaMemcpy(tmp.table, static_cast<const uint8_t *>(buf) + sizeof(ImageHeader), h.payload,
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gqf_sqf_free(&tmp);
        GQF_CK(e);
    }
    *qf = tmp;
    return GQF_OK;
}

int gqf_rsqf_load(gqf_rsqf *cqf, const void *buf, size_t len)
{
    if (!cqf) return GQF_ERR_ARG;
    ImageHeader h;
    int st = parse_image(RSQF_MAGIC, buf, len, h);
    if (st) return st;
    gqf_rsqf tmp;
    st = gqf_rsqf_init(&tmp, h.q);
    if (st) return st == GQF_ERR_ARG ? GQF_ERR_FORMAT : st;
    if (h.r != RSQF_R || h.unit != RSQF_BB || h.payload != (size_t)tmp.numBlocks * RSQF_BB) {
        gqf_rsqf_free(&tmp);
        return GQF_ERR_FORMAT;
    }
    cudaError_t e = cudaMemcpy(tmp.blocks, static_cast<const uint8_t *>(buf) + sizeof(ImageHeader), h.payload,
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gqf_rsqf_free(&tmp);
        GQF_CK(e);
    }
    *cqf = tmp;
    return GQF_OK;
}

int gqf_sqf_save_file(const gqf_sqf *qf, const char *path)
{
    if (!qf) return GQF_ERR_ARG;
    std::vector<uint8_t> v(gqf_sqf_image_bytes(qf));
    int st = gqf_sqf_save(qf, v.data(), v.size(), nullptr);
    return st ? st : write_file(path, v);
}

int gqf_rsqf_save_file(const gqf_rsqf *cqf, const char *path)
{
    if (!cqf) return GQF_ERR_ARG;
    std::vector<uint8_t> v(gqf_rsqf_image_bytes(cqf));
    int st = gqf_rsqf_save(cqf, v.data(), v.size(), nullptr);
    return st ? st : write_file(path, v);
}

int gqf_sqf_load_file(gqf_sqf *qf, const char *path)
{
    std::vector<uint8_t> v;
    int st = read_file(path, v);
    return st ? st : gqf_sqf_load(qf, v.data(), v.size());
}

int gqf_rsqf_load_file(gqf_rsqf *cqf, const char *path)
{
    std::vector<uint8_t> v;
    int st = read_file(path, v);
    return st ? st : gqf_rsqf_load(cqf, v.data(), v.size());
}

}  // extern "C"
