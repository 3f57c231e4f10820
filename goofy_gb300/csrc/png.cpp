// png.cpp -- PNG ingest: a PNG file in memory -> RGBA8 rows.
//
// The reference harness loads its test images with lodepng (Src/main.cpp:258-342,
// loadPngAsRgba8: lodepng::decode to 8-bit RGBA, alpha then forced to 255,
// width % 16 and height % 4 checked).  This decoder is written from the PNG
// specification (ISO/IEC 15948), DEFLATE (RFC 1951) and the zlib wrapper
// (RFC 1950): every colour type and bit depth, both interlace methods, chunk
// CRCs and the Adler-32 checksum verified.  The conversion to 8-bit RGBA uses
// the rules lodepng applies: 16-bit samples keep their high byte, grey levels
// of 1/2/4 bits scale by 255 / (2^depth - 1), a palette index past the
// palette gives opaque black, and tRNS makes the key colour (or each palette
// entry) transparent.  Width / height rules for the encoder stay with the
// caller, as they do in the harness.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "host_util.h"

namespace {

// ---- checksums -------------------------------------------------------------

const uint32_t* crc_table()
{
    static const struct Table {
        uint32_t t[256];
        Table()
        {
            for (uint32_t n = 0; n < 256; ++n) {
                uint32_t c = n;
                for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
                t[n] = c;
            }
        }
    } table;
    return table.t;
}

uint32_t crc32(const uint8_t* p, size_t n)
{
    const uint32_t* t = crc_table();
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; ++i) c = t[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

uint32_t adler32(const uint8_t* p, size_t n)
{
    uint32_t a = 1, b = 0;
    while (n) {
        const size_t k = n < 5552 ? n : 5552;  // largest run before b can pass 2^32
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521;
        b %= 65521;
        p += k;
        n -= k;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ---- DEFLATE ----------------------------------------------------------------

// LSB-first bit reader over the compressed stream; bits past the end read as
// zero and mark the reader bad once consumed.
class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}

    uint32_t peek(int k)
    {
        if (cnt_ < k) refill();
        return (uint32_t)(buf_ & ((1ull << k) - 1));
    }
    bool consume(int k)
    {
        if (cnt_ < k) {
            refill();
            if (cnt_ < k) {
                bad_ = true;
                buf_ = 0;
                cnt_ = 0;
                return false;
            }
        }
        buf_ >>= k;
        cnt_ -= k;
        return true;
    }
    uint32_t bits(int k)
    {
        const uint32_t v = peek(k);
        consume(k);
        return v;
    }
    void align()
    {
        const int drop = cnt_ & 7;
        buf_ >>= drop;
        cnt_ -= drop;
    }
    bool bad() const { return bad_; }

private:
    void refill()
    {
        while (cnt_ <= 56 && pos_ < n_) {
            buf_ |= (uint64_t)p_[pos_++] << cnt_;
            cnt_ += 8;
        }
    }
    const uint8_t* p_;
    size_t n_, pos_ = 0;
    uint64_t buf_ = 0;
    int cnt_ = 0;
    bool bad_ = false;
};

// Canonical Huffman code: a 10-bit direct table for short codes, a
// bit-at-a-time canonical walk for the longer ones.
struct Huffman {
    static constexpr int kFast = 10;
    uint16_t fast[1 << kFast];  // symbol | length << 9; 0 = no code of <= kFast bits
    uint16_t count[16];
    uint16_t symbol[320];

    bool build(const uint8_t* len, int n)
    {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; ++i) count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = 2 * left - count[l];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16] = {0};
        for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + count[l];
        uint32_t next[16] = {0};
        uint32_t code = 0;
        for (int l = 1; l < 16; ++l) {
            code = (code + count[l - 1]) << 1;
            next[l] = code;
        }
        std::memset(fast, 0, sizeof(fast));
        for (int i = 0; i < n; ++i) {
            const int l = len[i];
            if (!l) continue;
            symbol[offs[l]++] = (uint16_t)i;
            const uint32_t c = next[l]++;
            if (l <= kFast) {
                uint32_t r = 0;  // codes are sent most-significant bit first
                for (int b = 0; b < l; ++b) r |= ((c >> b) & 1) << (l - 1 - b);
                for (uint32_t j = r; j < (1u << kFast); j += 1u << l) fast[j] = (uint16_t)(i | l << 9);
            }
        }
        return true;
    }

    int decode(BitReader& br) const
    {
        const uint32_t v = br.peek(15);
        const uint16_t e = fast[v & ((1u << kFast) - 1)];
        if (e) return br.consume(e >> 9) ? (e & 511) : -1;
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (v >> (l - 1)) & 1;
            const int c = count[l];
            if (code - first < c) return br.consume(l) ? symbol[index + code - first] : -1;
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;  // bit pattern not assigned by an incomplete code
    }
};

struct Tables {
    uint16_t len_base[29], dist_base[30];
    uint8_t len_extra[29], dist_extra[30];
    Huffman fixed_lit, fixed_dist;
    Tables()
    {
        uint32_t b = 3;
        for (int s = 0; s < 28; ++s) {
            len_extra[s] = (uint8_t)(s < 8 ? 0 : (s - 4) / 4);
            len_base[s] = (uint16_t)b;
            b += 1u << len_extra[s];
        }
        len_base[28] = 258;
        len_extra[28] = 0;
        b = 1;
        for (int s = 0; s < 30; ++s) {
            dist_extra[s] = (uint8_t)(s < 4 ? 0 : (s - 2) / 2);
            dist_base[s] = (uint16_t)b;
            b += 1u << dist_extra[s];
        }
        uint8_t l[288];
        for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
        fixed_lit.build(l, 288);
        for (int i = 0; i < 30; ++i) l[i] = 5;
        fixed_dist.build(l, 30);
    }
};

const Tables& tables()
{
    static const Tables t;
    return t;
}

// zlib stream -> exactly `out_size` bytes, else an error message.
const char* inflate_zlib(const uint8_t* in, size_t n, uint8_t* out, size_t out_size)
{
    if (n < 6) return "zlib stream too short";
    const uint32_t cmf = in[0], flg = in[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0) return "bad zlib header";
    if (flg & 0x20) return "zlib preset dictionary not allowed in PNG";
    const Tables& T = tables();
    BitReader br(in + 2, n - 2);
    size_t o = 0;
    Huffman lit, dist;
    bool final_block = false;
    while (!final_block) {
        final_block = br.bits(1);
        const uint32_t type = br.bits(2);
        if (type == 0) {
            br.align();
            const uint32_t len = br.bits(16), nlen = br.bits(16);
            if ((len ^ 0xffffu) != nlen) return "stored block length check failed";
            if (len > out_size - o) return "more image data than the header allows";
            for (uint32_t i = 0; i < len; ++i) out[o++] = (uint8_t)br.bits(8);
            if (br.bad()) return "truncated stored block";
            continue;
        }
        const Huffman* L = &T.fixed_lit;
        const Huffman* D = &T.fixed_dist;
        if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            if (hlit > 286 || hdist > 30) return "too many length or distance codes";
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return "bad code-length code";
            uint8_t lens[320] = {0};
            for (int i = 0; i < hlit + hdist;) {
                const int sym = clh.decode(br);
                if (sym < 0) return "bad code-length symbol";
                if (sym < 16) {
                    lens[i++] = (uint8_t)sym;
                    continue;
                }
                int rep;
                uint8_t v = 0;
                if (sym == 16) {
                    if (i == 0) return "repeat with no previous length";
                    v = lens[i - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (i + rep > hlit + hdist) return "code lengths overrun";
                while (rep--) lens[i++] = v;
            }
            if (br.bad()) return "truncated block header";
            if (!lens[256]) return "no end-of-block code";
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return "over-subscribed Huffman code";
            L = &lit;
            D = &dist;
        } else if (type != 1) {
            return "bad block type";
        }
        for (;;) {
            const int sym = L->decode(br);
            if (sym < 0) return br.bad() ? "truncated compressed data" : "bad literal/length code";
            if (sym < 256) {
                if (o >= out_size) return "more image data than the header allows";
                out[o++] = (uint8_t)sym;
                continue;
            }
            if (sym == 256) break;
            const int ls = sym - 257;
            if (ls >= 29) return "bad length symbol";
            const uint32_t len = T.len_base[ls] + br.bits(T.len_extra[ls]);
            const int ds = D->decode(br);
            if (ds < 0 || ds >= 30) return "bad distance code";
            const uint32_t d = T.dist_base[ds] + br.bits(T.dist_extra[ds]);
            if (br.bad()) return "truncated compressed data";
            if (d > o) return "distance before the start of the data";
            if (len > out_size - o) return "more image data than the header allows";
            const uint8_t* s = out + o - d;
            for (uint32_t i = 0; i < len; ++i) out[o + i] = s[i];  // overlapping copies repeat the run
            o += len;
        }
    }
    br.align();
    uint32_t want = 0;
    for (int i = 0; i < 4; ++i) want = want << 8 | br.bits(8);
    if (br.bad()) return "missing Adler-32 checksum";
    if (o != out_size) return "less image data than the header needs";
    if (want != adler32(out, o)) return "Adler-32 checksum mismatch";
    return nullptr;
}

// ---- PNG --------------------------------------------------------------------

struct Png {
    uint32_t width = 0, height = 0;
    int depth = 0, ctype = 0, interlace = 0, channels = 0;
    uint8_t palette[256][4];
    int npal = 0;
    bool has_key = false;
    uint16_t key[3] = {0, 0, 0};
    std::vector<uint8_t> idat;
};

int bad(const char* what) { return goofy_gpu::fail(GOOFY_ERR_INVALID, what); }

int parse(const uint8_t* p, size_t n, Png& png, bool header_only)
{
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (!p || n < 8 + 25 || std::memcmp(p, sig, 8) != 0) return bad("png: not a PNG file");
    size_t pos = 8;
    bool seen_ihdr = false, seen_plte = false, seen_iend = false;
    while (pos + 12 <= n) {
        const uint32_t len = be32(p + pos);
        const uint8_t* type = p + pos + 4;
        const uint8_t* data = p + pos + 8;
        if (len > 0x7fffffffu || len > n - pos - 12) return bad("png: truncated chunk");
        if (crc32(type, (size_t)len + 4) != be32(data + len)) return bad("png: chunk CRC mismatch");
        pos += (size_t)len + 12;
        const bool is_ihdr = !std::memcmp(type, "IHDR", 4);
        if (seen_ihdr == is_ihdr) return bad(is_ihdr ? "png: second IHDR" : "png: IHDR is not the first chunk");
        if (is_ihdr) {
            if (len != 13) return bad("png: bad IHDR length");
            png.width = be32(data);
            png.height = be32(data + 4);
            png.depth = data[8];
            png.ctype = data[9];
            png.interlace = data[12];
            if (!png.width || !png.height || png.width > 0x7fffffffu || png.height > 0x7fffffffu)
                return bad("png: bad image size");
            const int d = png.depth;
            bool ok;
            switch (png.ctype) {
            case 0: ok = d == 1 || d == 2 || d == 4 || d == 8 || d == 16; png.channels = 1; break;
            case 2: ok = d == 8 || d == 16; png.channels = 3; break;
            case 3: ok = d == 1 || d == 2 || d == 4 || d == 8; png.channels = 1; break;
            case 4: ok = d == 8 || d == 16; png.channels = 2; break;
            case 6: ok = d == 8 || d == 16; png.channels = 4; break;
            default: ok = false;
            }
            if (!ok) return bad("png: bad colour type / bit depth");
            if (data[10] != 0 || data[11] != 0 || png.interlace > 1)
                return bad("png: unknown compression, filter or interlace method");
            seen_ihdr = true;
            if (header_only) return GOOFY_OK;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            if (len % 3 || len == 0 || len > 768) return bad("png: bad PLTE length");
            if (png.ctype == 0 || png.ctype == 4) return bad("png: PLTE in a grey image");
            png.npal = (int)len / 3;
            for (int i = 0; i < png.npal; ++i) {
                png.palette[i][0] = data[3 * i];
                png.palette[i][1] = data[3 * i + 1];
                png.palette[i][2] = data[3 * i + 2];
                png.palette[i][3] = 255;
            }
            seen_plte = true;
        } else if (!std::memcmp(type, "tRNS", 4)) {
            if (png.ctype == 3) {
                if (!seen_plte || (int)len > png.npal) return bad("png: bad tRNS for a palette image");
                for (uint32_t i = 0; i < len; ++i) png.palette[i][3] = data[i];
            } else if (png.ctype == 0 && len == 2) {
                png.has_key = true;
                png.key[0] = (uint16_t)(data[0] << 8 | data[1]);
            } else if (png.ctype == 2 && len == 6) {
                png.has_key = true;
                for (int c = 0; c < 3; ++c) png.key[c] = (uint16_t)(data[2 * c] << 8 | data[2 * c + 1]);
            } else {
                return bad("png: tRNS not allowed for this colour type");
            }
        } else if (!std::memcmp(type, "IDAT", 4)) {
            png.idat.insert(png.idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            seen_iend = true;
            break;
        } else if (!(type[0] & 0x20)) {
            return bad("png: unknown critical chunk");
        }
    }
    if (!seen_ihdr) return bad("png: no IHDR");
    if (!seen_iend) return bad("png: truncated file (no IEND)");
    if (png.ctype == 3 && !seen_plte) return bad("png: palette image without PLTE");
    if (png.idat.empty()) return bad("png: no image data");
    return GOOFY_OK;
}

struct Pass {
    uint32_t x0, y0, dx, dy, w, h;
};

// Sub-images in file order: one for a plain image, the seven Adam7 passes for
// an interlaced one (empty passes carry no bytes).
int passes(const Png& png, Pass out[7])
{
    if (!png.interlace) {
        out[0] = Pass{0, 0, 1, 1, png.width, png.height};
        return 1;
    }
    static const uint32_t a7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                      {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    for (int i = 0; i < 7; ++i) {
        const uint32_t x0 = a7[i][0], y0 = a7[i][1], dx = a7[i][2], dy = a7[i][3];
        const uint32_t w = png.width > x0 ? (png.width - x0 + dx - 1) / dx : 0;
        const uint32_t h = png.height > y0 ? (png.height - y0 + dy - 1) / dy : 0;
        out[i] = Pass{x0, y0, dx, dy, w, h};
    }
    return 7;
}

inline uint8_t paeth(int a, int b, int c)
{
    const int p = a + b - c;
    const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (uint8_t)(pa <= pb && pa <= pc ? a : pb <= pc ? b : c);
}

// Undo the scanline filters of one sub-image in place (filter byte + `rb` bytes per row).
bool unfilter(uint8_t* rows, uint32_t h, size_t rb, int bpp)
{
    const uint8_t* prev = nullptr;
    for (uint32_t y = 0; y < h; ++y) {
        uint8_t* f = rows + y * (rb + 1);
        uint8_t* cur = f + 1;
        switch (*f) {
        case 0: break;
        case 1:
            for (size_t i = bpp; i < rb; ++i) cur[i] = (uint8_t)(cur[i] + cur[i - bpp]);
            break;
        case 2:
            if (prev)
                for (size_t i = 0; i < rb; ++i) cur[i] = (uint8_t)(cur[i] + prev[i]);
            break;
        case 3:
            for (size_t i = 0; i < rb; ++i) {
                const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
                cur[i] = (uint8_t)(cur[i] + ((a + b) >> 1));
            }
            break;
        case 4:
            for (size_t i = 0; i < rb; ++i) {
                const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
                const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
                cur[i] = (uint8_t)(cur[i] + paeth(a, b, c));
            }
            break;
        default: return false;
        }
        prev = cur;
    }
    return true;
}

// One pixel of a row as RGBA8.
inline void to_rgba(const Png& png, const uint8_t* row, uint32_t x, uint8_t* o)
{
    const int d = png.depth;
    if (d < 8) {  // grey or palette, one sample packed most-significant bits first
        const uint32_t bit = x * (uint32_t)d;
        const uint32_t v = (row[bit >> 3] >> (8 - d - (bit & 7))) & ((1u << d) - 1);
        if (png.ctype == 3) {
            static const uint8_t black[4] = {0, 0, 0, 255};
            std::memcpy(o, (int)v < png.npal ? png.palette[v] : black, 4);
        } else {
            o[0] = o[1] = o[2] = (uint8_t)(v * 255 / ((1u << d) - 1));
            o[3] = (png.has_key && v == png.key[0]) ? 0 : 255;
        }
        return;
    }
    const int ch = png.channels;
    uint16_t s[4];
    if (d == 8) {
        for (int c = 0; c < ch; ++c) s[c] = row[x * ch + c];
    } else {
        for (int c = 0; c < ch; ++c) s[c] = (uint16_t)(row[2 * (x * ch + c)] << 8 | row[2 * (x * ch + c) + 1]);
    }
    const int shift = d == 16 ? 8 : 0;
    switch (png.ctype) {
    case 0:
        o[0] = o[1] = o[2] = (uint8_t)(s[0] >> shift);
        o[3] = (png.has_key && s[0] == png.key[0]) ? 0 : 255;
        break;
    case 2:
        for (int c = 0; c < 3; ++c) o[c] = (uint8_t)(s[c] >> shift);
        o[3] = (png.has_key && s[0] == png.key[0] && s[1] == png.key[1] && s[2] == png.key[2]) ? 0 : 255;
        break;
    case 3: {
        static const uint8_t black[4] = {0, 0, 0, 255};
        std::memcpy(o, (int)s[0] < png.npal ? png.palette[s[0]] : black, 4);
        break;
    }
    case 4:
        o[0] = o[1] = o[2] = (uint8_t)(s[0] >> shift);
        o[3] = (uint8_t)(s[1] >> shift);
        break;
    default:
        for (int c = 0; c < 4; ++c) o[c] = (uint8_t)(s[c] >> shift);
    }
}

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_png_info(const void* png_bytes, size_t size, uint32_t* width, uint32_t* height)
{
    if (!width || !height) return GOOFY_ERR_INVALID;
    Png png;
    const int rc = parse(static_cast<const uint8_t*>(png_bytes), size, png, true);
    if (rc != GOOFY_OK) return rc;
    *width = png.width;
    *height = png.height;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_png_decode(const void* png_bytes, size_t size, void* rgba, size_t rgba_bytes,
                                      uint32_t stride, int opaque, uint32_t* width, uint32_t* height)
{
    Png png;
    int rc = parse(static_cast<const uint8_t*>(png_bytes), size, png, false);
    if (rc != GOOFY_OK) return rc;
    if (width) *width = png.width;
    if (height) *height = png.height;
    if (!rgba || (uint64_t)stride < 4ull * png.width) return goofy_gpu::fail(GOOFY_ERR_INVALID, "png: stride < 4*width");
    if ((uint64_t)stride * (png.height - 1) + 4ull * png.width > rgba_bytes)
        return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "png: output buffer too small");
    Pass ps[7];
    const int np = passes(png, ps);
    const int bits_pp = png.depth * png.channels;
    size_t total = 0;
    for (int i = 0; i < np; ++i)
        if (ps[i].w && ps[i].h) total += (size_t)ps[i].h * (((size_t)ps[i].w * bits_pp + 7) / 8 + 1);
    std::vector<uint8_t> raw;
    try {
        raw.resize(total);
    } catch (...) {
        return goofy_gpu::fail(GOOFY_ERR_NOMEM, "png: out of host memory");
    }
    if (const char* err = inflate_zlib(png.idat.data(), png.idat.size(), raw.data(), total)) {
        static thread_local char msg[96];
        std::snprintf(msg, sizeof(msg), "png: %s", err);
        return bad(msg);
    }
    const int bpp = bits_pp >= 8 ? bits_pp / 8 : 1;
    uint8_t* base = static_cast<uint8_t*>(rgba);
    size_t off = 0;
    for (int i = 0; i < np; ++i) {
        const Pass& p = ps[i];
        if (!p.w || !p.h) continue;
        const size_t rb = ((size_t)p.w * bits_pp + 7) / 8;
        uint8_t* rows = raw.data() + off;
        if (!unfilter(rows, p.h, rb, bpp)) return bad("png: bad filter type");
        for (uint32_t y = 0; y < p.h; ++y) {
            const uint8_t* row = rows + y * (rb + 1) + 1;
            uint8_t* o = base + (size_t)(p.y0 + y * p.dy) * stride + 4 * (size_t)p.x0;
            if (png.ctype == 6 && png.depth == 8 && p.dx == 1) {
                std::memcpy(o, row, 4 * (size_t)p.w);
            } else {
                for (uint32_t x = 0; x < p.w; ++x) to_rgba(png, row, x, o + 4 * (size_t)x * p.dx);
            }
            if (opaque)
                for (uint32_t x = 0; x < p.w; ++x) o[4 * (size_t)x * p.dx + 3] = 255;
        }
        off += (size_t)p.h * (rb + 1);
    }
    return GOOFY_OK;
}

}  // extern "C"
