// cr_image.cpp -- image files of the film and of textures, the behaviour of
// Image (Utils/Image.cpp) with codecs written here:
//   - EXR write, Image::writeEXR (:49-106): B, G, R channels (the order EXR
//     readers expect), HALF pixels, uncompressed scanlines, as tinyexr
//     serialises it; its float -> half conversion rounds a dropped half-ulp up
//     in magnitude (the ISPC reference conversion tinyexr uses);
//   - EXR read, Image::readEXR (:108-180): single-part scanline files with
//     NONE / RLE / ZIPS / ZIP compression and HALF / FLOAT / UINT channels;
//     R, G, B are the first channels whose names start with those letters,
//     further channels are kept as zeros;
//   - PNG write, Image::writePNG (:182-217): 8 bits per channel, values
//     optionally gamma-encoded (pow 1/2.2) and clamped, then truncated;
//   - PNG read, Image::readMisc (:219-260): 8/16-bit grey, RGB, RGBA and
//     palette images, rows flipped to bottom-up as stb's
//     flip-vertically-on-load does, values / 255 and, for textures, raised
//     to the power 2.2.
// zlib (RFC 1950/1951), CRC-32 and the PNG filters follow their
// specifications; the EXR layout follows the OpenEXR file format document.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "craystal_c.h"
#include "cr_io.h"

namespace cr {
namespace io {

// ---------------------------------------------------------------------------
// checksums
// ---------------------------------------------------------------------------
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

static uint32_t crc32Update(uint32_t crc, const uint8_t* p, size_t n) {
    static const CrcTable table;  // initialised once, thread-safe
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

static uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; i++) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

// ---------------------------------------------------------------------------
// inflate (RFC 1951), canonical Huffman codes decoded bit by bit
// ---------------------------------------------------------------------------
namespace {

struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t bitBuf = 0;
    int bitCnt = 0;
    bool bad = false;
    int bit() {
        if (bitCnt == 0) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            bitBuf = p[pos++];
            bitCnt = 8;
        }
        const int b = bitBuf & 1;
        bitBuf >>= 1;
        bitCnt--;
        return b;
    }
    uint32_t bits(int k) {
        uint32_t v = 0;
        for (int i = 0; i < k; i++) v |= (uint32_t)bit() << i;
        return v;
    }
};

struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
    bool build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++) offs[len + 1] = offs[len] + count[len];
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= br.bit();
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (br.bad) return -1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6,
                                7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflateCodes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    while (true) {
        const int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) return false;
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int di = dist.decode(br);
            if (di < 0 || di >= 30) return false;
            const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
            if (br.bad || d > out.size()) return false;
            const size_t start = out.size() - d;
            for (size_t k = 0; k < len; k++) out.push_back(out[start + k]);
        }
    }
}

struct FixedCodes {
    Huffman lit, dist;
    FixedCodes() {
        uint8_t l[288];
        for (int i = 0; i < 144; i++) l[i] = 8;
        for (int i = 144; i < 256; i++) l[i] = 9;
        for (int i = 256; i < 280; i++) l[i] = 7;
        for (int i = 280; i < 288; i++) l[i] = 8;
        lit.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; i++) d[i] = 5;
        dist.build(d, 30);
    }
};

}  // namespace

bool inflateRaw(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
    BitReader br{p, n};
    int last = 0;
    do {
        last = br.bit();
        const uint32_t type = br.bits(2);
        if (br.bad) return false;
        if (type == 0) {  // stored
            br.bitCnt = 0;
            if (br.pos + 4 > n) return false;
            const uint32_t len = p[br.pos] | (p[br.pos + 1] << 8);
            const uint32_t nlen = p[br.pos + 2] | (p[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || br.pos + len > n) return false;
            out.insert(out.end(), p + br.pos, p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {  // fixed codes
            static const FixedCodes fixed;  // initialised once, thread-safe
            if (!inflateCodes(br, fixed.lit, fixed.dist, out)) return false;
        } else if (type == 2) {  // dynamic codes
            const int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
            if (nlen > 286 || ndist > 30) return false;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t lengths[320] = {0};
            for (int i = 0; i < ncode; i++) lengths[order[i]] = (uint8_t)br.bits(3);
            Huffman lencode;
            if (!lencode.build(lengths, 19)) return false;
            int idx = 0;
            while (idx < nlen + ndist) {
                const int sym = lencode.decode(br);
                if (sym < 0) return false;
                if (sym < 16) {
                    lengths[idx++] = (uint8_t)sym;
                } else {
                    uint8_t v = 0;
                    int rep;
                    if (sym == 16) {
                        if (idx == 0) return false;
                        v = lengths[idx - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (idx + rep > nlen + ndist) return false;
                    while (rep--) lengths[idx++] = v;
                }
            }
            if (lengths[256] == 0) return false;
            Huffman lit, dist;
            if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist)) return false;
            if (!inflateCodes(br, lit, dist, out)) return false;
        } else {
            return false;
        }
        if (br.bad) return false;
    } while (!last);
    return true;
}

bool zlibDecompress(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
    if (n < 6) return false;
    const uint8_t cmf = p[0], flg = p[1];
    if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
    const size_t before = out.size();
    if (!inflateRaw(p + 2, n - 6, out)) return false;
    const uint32_t want = ((uint32_t)p[n - 4] << 24) | ((uint32_t)p[n - 3] << 16) | ((uint32_t)p[n - 2] << 8) | p[n - 1];
    return adler32(out.data() + before, out.size() - before) == want;
}

// zlib stream of stored (uncompressed) deflate blocks
static void zlibStore(const std::vector<uint8_t>& raw, std::vector<uint8_t>& out) {
    out.push_back(0x78);
    out.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        out.push_back(last ? 1 : 0);
        out.push_back((uint8_t)(len & 0xFF));
        out.push_back((uint8_t)(len >> 8));
        out.push_back((uint8_t)(~len & 0xFF));
        out.push_back((uint8_t)((~len >> 8) & 0xFF));
        out.insert(out.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    const uint32_t a = adler32(raw.data(), raw.size());
    for (int s = 24; s >= 0; s -= 8) out.push_back((uint8_t)(a >> s));
}

// ---------------------------------------------------------------------------
// half floats
// ---------------------------------------------------------------------------
// float -> half as tinyexr converts (ISPC reference code): truncate the
// mantissa and add one unit when the first dropped bit is set (ties round
// up in magnitude); overflow gives infinity, NaN a quiet NaN.
uint16_t floatToHalf(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t sign = (u >> 16) & 0x8000u;
    const int exp = (int)((u >> 23) & 0xFF);
    const uint32_t mant = u & 0x7FFFFFu;
    uint32_t h = 0;
    if (exp == 0) {
        h = 0;
    } else if (exp == 255) {
        h = (31u << 10) | (mant ? 0x200u : 0u);
    } else {
        const int e = exp - 127 + 15;
        if (e >= 31) {
            h = 31u << 10;
        } else if (e <= 0) {
            if (14 - e <= 24) {
                const uint32_t m = mant | 0x800000u;
                h = m >> (14 - e);
                if ((m >> (13 - e)) & 1u) h++;
            }
        } else {
            h = ((uint32_t)e << 10) | (mant >> 13);
            if (mant & 0x1000u) h++;
        }
    }
    return (uint16_t)(h | sign);
}

float halfToFloat(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1Fu;
    uint32_t mant = h & 0x3FFu;
    uint32_t u;
    if (exp == 0) {
        if (mant == 0) {
            u = sign;
        } else {  // subnormal half -> normal float
            int e = -1;
            do {
                e++;
                mant <<= 1;
            } while (!(mant & 0x400u));
            u = sign | ((uint32_t)(127 - 15 - e) << 23) | ((mant & 0x3FFu) << 13);
        }
    } else if (exp == 31) {
        u = sign | 0x7F800000u | (mant << 13);
    } else {
        u = sign | ((exp + 127 - 15) << 23) | (mant << 13);
    }
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// ---------------------------------------------------------------------------
// files
// ---------------------------------------------------------------------------
bool readFile(const std::string& path, std::vector<uint8_t>& data) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        return false;
    }
    data.resize((size_t)n);
    const size_t got = n ? std::fread(data.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == (size_t)n;
}

static bool writeFile(const std::string& path, const std::vector<uint8_t>& data) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t put = std::fwrite(data.data(), 1, data.size(), f);
    return std::fclose(f) == 0 && put == data.size();
}

static void put32(std::vector<uint8_t>& v, uint32_t x) {  // little endian
    for (int k = 0; k < 4; k++) v.push_back((uint8_t)(x >> (8 * k)));
}
static void put64(std::vector<uint8_t>& v, uint64_t x) {
    for (int k = 0; k < 8; k++) v.push_back((uint8_t)(x >> (8 * k)));
}
static void putStr(std::vector<uint8_t>& v, const char* s) { v.insert(v.end(), s, s + std::strlen(s) + 1); }
static void putAttr(std::vector<uint8_t>& v, const char* name, const char* type, const std::vector<uint8_t>& val) {
    putStr(v, name);
    putStr(v, type);
    put32(v, (uint32_t)val.size());
    v.insert(v.end(), val.begin(), val.end());
}
static uint32_t get32(const uint8_t* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
static uint64_t get64(const uint8_t* p) { return get32(p) | ((uint64_t)get32(p + 4) << 32); }
static uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | (p[1] << 16) | (p[2] << 8) | p[3]; }

// ---------------------------------------------------------------------------
// EXR
// ---------------------------------------------------------------------------
int writeExr(const std::string& path, uint32_t w, uint32_t h, uint32_t ch, const float* px, std::string& err) {
    if (ch < 3) {
        err = "an EXR film needs at least 3 channels";
        return CR_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> f = {0x76, 0x2f, 0x31, 0x01};
    put32(f, 2);
    static const char* names[3] = {"B", "G", "R"};
    std::vector<uint8_t> chl;
    for (const char* nm : names) {
        putStr(chl, nm);
        put32(chl, 1);  // HALF
        chl.push_back(0);  // pLinear
        chl.push_back(0);
        chl.push_back(0);
        chl.push_back(0);
        put32(chl, 1);
        put32(chl, 1);
    }
    chl.push_back(0);
    putAttr(f, "channels", "chlist", chl);
    putAttr(f, "compression", "compression", {0});
    std::vector<uint8_t> box;
    put32(box, 0);
    put32(box, 0);
    put32(box, w - 1);
    put32(box, h - 1);
    putAttr(f, "dataWindow", "box2i", box);
    putAttr(f, "displayWindow", "box2i", box);
    putAttr(f, "lineOrder", "lineOrder", {0});
    std::vector<uint8_t> one;
    const float fone = 1.0f, fzero = 0.0f;
    uint32_t bits;
    std::memcpy(&bits, &fone, 4);
    put32(one, bits);
    putAttr(f, "pixelAspectRatio", "float", one);
    std::vector<uint8_t> center;
    std::memcpy(&bits, &fzero, 4);
    put32(center, bits);
    put32(center, bits);
    putAttr(f, "screenWindowCenter", "v2f", center);
    putAttr(f, "screenWindowWidth", "float", one);
    f.push_back(0);
    const size_t table = f.size();
    const size_t lineBytes = 3 * 2 * (size_t)w;
    for (uint32_t y = 0; y < h; y++) put64(f, table + 8 * (uint64_t)h + (uint64_t)y * (8 + lineBytes));
    for (uint32_t y = 0; y < h; y++) {
        put32(f, y);
        put32(f, (uint32_t)lineBytes);
        for (int c = 2; c >= 0; c--)  // B, G, R
            for (uint32_t x = 0; x < w; x++) {
                const uint16_t hv = floatToHalf(px[((size_t)y * w + x) * ch + c]);
                f.push_back((uint8_t)(hv & 0xFF));
                f.push_back((uint8_t)(hv >> 8));
            }
    }
    if (!writeFile(path, f)) {
        err = "cannot write " + path;
        return CR_ERR_IO;
    }
    return CR_OK;
}

namespace {

struct ExrChannel {
    std::string name;
    int type;  // 0 UINT, 1 HALF, 2 FLOAT
};

// ZIP / RLE post-processing of OpenEXR: the bytes were split into even and
// odd halves and delta-coded before compression.
void exrUnpredict(std::vector<uint8_t>& t, std::vector<uint8_t>& out) {
    for (size_t i = 1; i < t.size(); i++) t[i] = (uint8_t)(t[i - 1] + t[i] - 128);
    out.resize(t.size());
    const size_t half = (t.size() + 1) / 2;
    for (size_t i = 0; i < t.size(); i++) out[i] = (i & 1) ? t[half + i / 2] : t[i / 2];
}

bool exrRle(const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
    size_t i = 0;
    while (i < n) {
        const int8_t c = (int8_t)p[i++];
        if (c < 0) {
            const size_t cnt = (size_t)(-c);
            if (i + cnt > n) return false;
            out.insert(out.end(), p + i, p + i + cnt);
            i += cnt;
        } else {
            if (i >= n) return false;
            out.insert(out.end(), (size_t)c + 1, p[i++]);
        }
    }
    return true;
}

}  // namespace

int readExr(const std::vector<uint8_t>& d, Image& img, std::string& err) {
    auto bad = [&](const char* why) {
        err = std::string("EXR: ") + why;
        return CR_ERR_IO;
    };
    if (d.size() < 8 || get32(d.data()) != 20000630u) return bad("not an OpenEXR file");
    const uint32_t ver = get32(d.data() + 4);
    if ((ver & 0xFF) != 2) return bad("unsupported version");
    if (ver & 0x1A00u) {
        err = "EXR: tiled, deep or multi-part files are not supported";
        return CR_ERR_UNSUPPORTED;
    }
    size_t pos = 8;
    std::vector<ExrChannel> chans;
    int compression = -1;
    int32_t xmin = 0, ymin = 0, xmax = -1, ymax = -1;
    while (true) {
        if (pos >= d.size()) return bad("truncated header");
        if (d[pos] == 0) {
            pos++;
            break;
        }
        const std::string name((const char*)&d[pos]);
        pos += name.size() + 1;
        if (pos >= d.size()) return bad("truncated header");
        const std::string type((const char*)&d[pos]);
        pos += type.size() + 1;
        if (pos + 4 > d.size()) return bad("truncated header");
        const uint32_t size = get32(&d[pos]);
        pos += 4;
        if (pos + size > d.size()) return bad("truncated attribute");
        const uint8_t* v = &d[pos];
        if (name == "channels") {
            size_t q = 0;
            while (q < size && v[q] != 0) {
                ExrChannel c;
                c.name = std::string((const char*)v + q);
                q += c.name.size() + 1;
                if (q + 16 > size) return bad("bad channel list");
                c.type = (int)get32(v + q);
                if (c.type < 0 || c.type > 2) return bad("bad pixel type");
                if (get32(v + q + 8) != 1 || get32(v + q + 12) != 1) {
                    err = "EXR: subsampled channels are not supported";
                    return CR_ERR_UNSUPPORTED;
                }
                q += 16;
                chans.push_back(c);
            }
        } else if (name == "compression") {
            compression = v[0];
        } else if (name == "dataWindow") {
            xmin = (int32_t)get32(v);
            ymin = (int32_t)get32(v + 4);
            xmax = (int32_t)get32(v + 8);
            ymax = (int32_t)get32(v + 12);
        }
        pos += size;
    }
    if (chans.empty() || xmax < xmin || ymax < ymin) return bad("missing channels or data window");
    int lpb;
    switch (compression) {
        case 0:
        case 1:
        case 2:
            lpb = 1;
            break;
        case 3:
            lpb = 16;
            break;
        default:
            err = "EXR: compression " + std::to_string(compression) + " is not supported (NONE, RLE, ZIPS, ZIP are)";
            return CR_ERR_UNSUPPORTED;
    }
    // Image::readEXR maps R, G, B to the first channel whose name starts with the letter
    int map[3];
    for (int i = 0; i < 3; i++) {
        map[i] = -1;
        for (size_t j = 0; j < chans.size(); j++)
            if (!chans[j].name.empty() && chans[j].name[0] == "RGB"[i]) {
                map[i] = (int)j;
                break;
            }
        if (map[i] < 0) return bad("no R, G and B channels");
    }
    const uint32_t w = (uint32_t)(xmax - xmin + 1), h = (uint32_t)(ymax - ymin + 1);
    img.width = w;
    img.height = h;
    img.channels = (uint32_t)std::max<size_t>(3, chans.size());
    img.pixels.assign((size_t)w * h * img.channels, 0.0f);
    size_t lineBytes = 0;
    for (const ExrChannel& c : chans) lineBytes += (size_t)w * (c.type == 1 ? 2 : 4);
    const uint32_t nBlocks = (h + lpb - 1) / lpb;
    if (pos + 8 * (size_t)nBlocks > d.size()) return bad("truncated offset table");
    std::vector<uint8_t> raw, tmp;
    for (uint32_t b = 0; b < nBlocks; b++) {
        const uint64_t off = get64(&d[pos + 8 * (size_t)b]);
        if (off + 8 > d.size()) return bad("bad block offset");
        const int32_t y0 = (int32_t)get32(&d[off]);
        const uint32_t size = get32(&d[off + 4]);
        if (off + 8 + size > d.size()) return bad("truncated block");
        const uint8_t* src = &d[off + 8];
        if (y0 < ymin || y0 > ymax) return bad("block outside the data window");
        const uint32_t lines = std::min<uint32_t>(lpb, (uint32_t)(ymax - y0 + 1));
        const size_t want = lineBytes * lines;
        const uint8_t* data = src;
        if (compression != 0 && size < want) {  // compressed block (stored raw when that is no smaller)
            raw.clear();
            tmp.clear();
            bool ok;
            if (compression == 1) {
                ok = exrRle(src, size, tmp);
            } else {
                ok = zlibDecompress(src, size, tmp);
            }
            if (!ok || (compression != 0 && tmp.size() != want)) return bad("corrupt compressed block");
            exrUnpredict(tmp, raw);
            data = raw.data();
        } else if (size != want) {
            return bad("block size");
        }
        for (uint32_t l = 0; l < lines; l++) {
            const uint32_t y = (uint32_t)(y0 - ymin) + l;
            const uint8_t* q = data + l * lineBytes;
            for (size_t j = 0; j < chans.size(); j++) {
                const int type = chans[j].type;
                const int bytes = type == 1 ? 2 : 4;
                int dst = -1;
                for (int i = 0; i < 3; i++)
                    if (map[i] == (int)j) dst = i;
                if (dst >= 0)
                    for (uint32_t x = 0; x < w; x++) {
                        const uint8_t* s = q + (size_t)x * bytes;
                        float v;
                        if (type == 1) {
                            v = halfToFloat((uint16_t)(s[0] | (s[1] << 8)));
                        } else if (type == 2) {
                            const uint32_t u = get32(s);
                            std::memcpy(&v, &u, 4);
                        } else {
                            v = (float)get32(s);
                        }
                        img.pixels[((size_t)y * w + x) * img.channels + dst] = v;
                    }
                q += (size_t)w * bytes;
            }
        }
    }
    return CR_OK;
}

// ---------------------------------------------------------------------------
// PNG
// ---------------------------------------------------------------------------
// float -> unsigned char as the reference's x86 build converts it: the
// value truncates to a 32-bit integer (NaN and out-of-range values become
// INT_MIN) whose low byte is kept.
static uint8_t toByteX86(float v) {
    int32_t i;
    if (!(v > -2147483648.0f && v < 2147483648.0f)) {
        i = INT32_MIN;
    } else {
        i = (int32_t)v;
    }
    return (uint8_t)(i & 0xFF);
}

int writePng(const std::string& path, uint32_t w, uint32_t h, uint32_t ch, const float* px, bool gamma,
             std::string& err) {
    if (ch < 1 || ch > 4) {
        err = "PNG images have 1 to 4 channels";
        return CR_ERR_INVALID_ARGUMENT;
    }
    static const uint8_t colorType[5] = {0, 0, 4, 2, 6};
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (1 + (size_t)w * ch));
    for (uint32_t y = 0; y < h; y++) {
        raw.push_back(0);  // filter: none
        for (size_t i = 0; i < (size_t)w * ch; i++) {
            float v = px[(size_t)y * w * ch + i];
            if (gamma) {  // Linear colour space: pow(v, 1 / 2.2), then saturate
                v = std::pow(v, 1.0f / 2.2f);
                v = v < 0.0f ? 0.0f : (1.0f < v ? 1.0f : v);
            }
            raw.push_back(toByteX86(v * 255.f));
        }
    }
    std::vector<uint8_t> f = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    auto chunk = [&](const char* type, const std::vector<uint8_t>& body) {
        const uint32_t n = (uint32_t)body.size();
        for (int s = 24; s >= 0; s -= 8) f.push_back((uint8_t)(n >> s));
        const size_t start = f.size();
        f.insert(f.end(), type, type + 4);
        f.insert(f.end(), body.begin(), body.end());
        const uint32_t crc = crc32Update(0, &f[start], 4 + body.size());
        for (int s = 24; s >= 0; s -= 8) f.push_back((uint8_t)(crc >> s));
    };
    std::vector<uint8_t> ihdr;
    for (uint32_t v : {w, h})
        for (int s = 24; s >= 0; s -= 8) ihdr.push_back((uint8_t)(v >> s));
    ihdr.insert(ihdr.end(), {8, colorType[ch], 0, 0, 0});
    chunk("IHDR", ihdr);
    std::vector<uint8_t> z;
    zlibStore(raw, z);
    chunk("IDAT", z);
    chunk("IEND", {});
    if (!writeFile(path, f)) {
        err = "cannot write " + path;
        return CR_ERR_IO;
    }
    return CR_OK;
}

static int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

int readPng(const std::vector<uint8_t>& d, bool toLinear, Image& img, std::string& err) {
    auto bad = [&](const char* why) {
        err = std::string("PNG: ") + why;
        return CR_ERR_IO;
    };
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0) return bad("not a PNG file");
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette, trns;
    while (pos + 12 <= d.size()) {
        const uint32_t n = be32(&d[pos]);
        const std::string type((const char*)&d[pos + 4], 4);
        if (pos + 12 + (size_t)n > d.size()) return bad("truncated chunk");
        const uint8_t* body = &d[pos + 8];
        if (type == "IHDR") {
            if (n < 13) return bad("short IHDR");
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
        } else if (type == "PLTE") {
            palette.assign(body, body + n);
        } else if (type == "tRNS") {
            trns.assign(body, body + n);
        } else if (type == "IDAT") {
            idat.insert(idat.end(), body, body + n);
        } else if (type == "IEND") {
            break;
        }
        pos += 12 + n;
    }
    if (w == 0 || h == 0 || ctype < 0) return bad("missing header");
    if (interlace) {
        err = "PNG: interlaced images are not supported";
        return CR_ERR_UNSUPPORTED;
    }
    int inCh;
    switch (ctype) {
        case 0: inCh = 1; break;
        case 2: inCh = 3; break;
        case 3: inCh = 1; break;
        case 4: inCh = 2; break;
        case 6: inCh = 4; break;
        default: return bad("bad colour type");
    }
    if (ctype == 4) {  // Image::readMisc accepts 1, 3 and 4 channels only
        err = "PNG: unsupported colour type (grey + alpha)";
        return CR_ERR_UNSUPPORTED;
    }
    if (!(depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4))))
        return bad("bad bit depth");
    if (ctype == 3 && (depth == 16 || palette.empty())) return bad("bad palette");
    std::vector<uint8_t> raw;
    if (!zlibDecompress(idat.data(), idat.size(), raw)) return bad("corrupt image data");
    const size_t bitsPerPx = (size_t)inCh * depth;
    const size_t stride = ((size_t)w * bitsPerPx + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bitsPerPx / 8);
    if (raw.size() < h * (stride + 1)) return bad("short image data");
    std::vector<uint8_t> rows((size_t)h * stride), prev(stride, 0);
    for (uint32_t y = 0; y < h; y++) {
        const uint8_t ft = raw[y * (stride + 1)];
        const uint8_t* src = &raw[y * (stride + 1) + 1];
        uint8_t* cur = &rows[(size_t)y * stride];
        for (size_t i = 0; i < stride; i++) {
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            int v = src[i];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return bad("bad filter");
            }
            cur[i] = (uint8_t)v;
        }
        std::memcpy(prev.data(), cur, stride);
    }
    const bool palAlpha = ctype == 3 && !trns.empty();
    const uint32_t outCh = ctype == 3 ? (palAlpha ? 4u : 3u) : (uint32_t)inCh;
    img.width = w;
    img.height = h;
    img.channels = outCh;
    img.pixels.assign((size_t)w * h * outCh, 0.0f);
    const int scale = depth == 1 ? 255 : depth == 2 ? 85 : depth == 4 ? 17 : 1;
    for (uint32_t y = 0; y < h; y++) {
        const uint8_t* r = &rows[(size_t)y * stride];
        const uint32_t dy = h - 1 - y;  // flipped vertically on load
        for (uint32_t x = 0; x < w; x++) {
            uint8_t px[4] = {0, 0, 0, 255};
            if (depth < 8) {
                const size_t bit = (size_t)x * depth;
                const int v = (r[bit / 8] >> (8 - depth - (int)(bit % 8))) & ((1 << depth) - 1);
                if (ctype == 3) {
                    if ((size_t)v * 3 + 2 >= palette.size()) return bad("palette index");
                    for (int k = 0; k < 3; k++) px[k] = palette[3 * v + k];
                    px[3] = (size_t)v < trns.size() ? trns[v] : 255;
                } else {
                    px[0] = (uint8_t)(v * scale);
                }
            } else if (ctype == 3) {
                const int v = r[x];
                if ((size_t)v * 3 + 2 >= palette.size()) return bad("palette index");
                for (int k = 0; k < 3; k++) px[k] = palette[3 * v + k];
                px[3] = (size_t)v < trns.size() ? trns[v] : 255;
            } else {
                for (int k = 0; k < inCh; k++)
                    px[k] = depth == 8 ? r[(size_t)x * inCh + k] : r[((size_t)x * inCh + k) * 2];  // 16 -> 8: high byte
            }
            for (uint32_t k = 0; k < outCh; k++) {
                float v = float(px[k]) / 255.f;
                if (toLinear) v = (float)std::pow((double)v, 2.2);
                img.pixels[((size_t)dy * w + x) * outCh + k] = v;
            }
        }
    }
    return CR_OK;
}

int loadImage(const std::string& path, bool toLinear, Image& img, std::string& err) {
    std::vector<uint8_t> d;
    if (!readFile(path, d)) {
        err = "cannot read " + path;
        return CR_ERR_IO;
    }
    const size_t dot = path.find_last_of('.');
    const std::string ext = dot == std::string::npos ? "" : path.substr(dot);
    if (ext == ".exr") return readExr(d, img, err);  // Image::load: EXR by extension, the rest through stb
    if (d.size() >= 8 && d[0] == 0x89 && d[1] == 'P' && d[2] == 'N' && d[3] == 'G') return readPng(d, toLinear, img, err);
    err = "unsupported image format: " + path + " (PNG and EXR are read)";
    return CR_ERR_UNSUPPORTED;
}

}  // namespace io
}  // namespace cr
