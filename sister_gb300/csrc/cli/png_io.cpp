// Minimal PNG reader / writer (see png_io.h).
#include "png_io.h"

#include <cstdio>
#include <cstring>

namespace pngio {
namespace {

// ---------------------------------------------------------------- DEFLATE decoder (RFC 1951)
// Bit reader: DEFLATE packs data LSB first. peek() looks at the next k bits (zero past the end of the input),
// skip() consumes them and flags a read past the end.
struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool bad = false;
    void fill() {
        while (cnt <= 56 && pos < n) {
            buf |= (uint64_t)p[pos++] << cnt;
            cnt += 8;
        }
    }
    unsigned peek(int k) {
        if (cnt < k) fill();
        return (unsigned)(buf & ((1ull << k) - 1));
    }
    void skip(int k) {
        if (cnt < k) fill();
        if (cnt < k) {
            bad = true;
            buf = 0;
            cnt = 0;
            return;
        }
        buf >>= k;
        cnt -= k;
    }
    int need(int k) { // the next k bits as a number, consumed
        if (k == 0) return 0;
        const int v = (int)peek(k);
        skip(k);
        return bad ? 0 : v;
    }
    size_t byte_end() const { return pos - (size_t)(cnt >> 3); } // first byte not touched by consumed bits
    void align() { // drop the bits of the current byte (stored blocks start on a byte boundary)
        const int drop = cnt & 7;
        buf >>= drop;
        cnt -= drop;
    }
};

// Huffman decoding by direct lookup: the table is indexed by the next kMaxBits input bits and holds, for
// every index, the symbol whose (bit-reversed) canonical code is a prefix of those bits and the code's length.
// Canonical codes follow RFC 1951 section 3.2.2: codes of each length are consecutive, shorter codes first,
// in symbol order within a length.
constexpr int kMaxBits = 15;
struct Huff {
    std::vector<uint32_t> table; // (symbol << 4) | length; 0 = no code (invalid input)
};

unsigned reverse_bits(unsigned v, int len) {
    unsigned r = 0;
    for (int k = 0; k < len; k++) r |= ((v >> k) & 1u) << (len - 1 - k);
    return r;
}

// false for an over-subscribed set of lengths (incomplete sets are accepted, as zlib does for one-code trees)
bool build(Huff &h, const int *len, int n) {
    int count[kMaxBits + 1] = {};
    for (int s = 0; s < n; s++) count[len[s]]++;
    count[0] = 0;
    long kraft = 0; // sum of 2^(kMaxBits - length)
    for (int l = 1; l <= kMaxBits; l++) kraft += (long)count[l] << (kMaxBits - l);
    if (kraft > (1L << kMaxBits)) return false;
    unsigned next[kMaxBits + 2] = {};
    unsigned code = 0;
    for (int l = 1; l <= kMaxBits; l++) {
        code = (code + count[l - 1]) << 1;
        next[l] = code;
    }
    h.table.assign(1u << kMaxBits, 0u);
    for (int s = 0; s < n; s++) {
        const int l = len[s];
        if (!l) continue;
        const unsigned r = reverse_bits(next[l]++, l);
        for (unsigned hi = 0; hi < (1u << (kMaxBits - l)); hi++) h.table[r | (hi << l)] = (uint32_t)s << 4 | (uint32_t)l;
    }
    return true;
}

int decode(Bits &b, const Huff &h) {
    const uint32_t e = h.table[b.peek(kMaxBits)];
    if (!e) return -1;
    b.skip((int)(e & 15u));
    return b.bad ? -1 : (int)(e >> 4);
}

// the fixed codes of block type 1 (RFC 1951 section 3.2.6), built once (thread-safe static initialisation)
struct FixedCodes {
    Huff lit, dist;
    FixedCodes() {
        int l[288], d[30];
        for (int s = 0; s < 288; s++) l[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
        for (int s = 0; s < 30; s++) d[s] = 5;
        build(lit, l, 288);
        build(dist, d, 30);
    }
};

const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131,
                          163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537,
                           2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12,
                            13, 13};

std::string codes(Bits &b, const Huff &lit, const Huff &dist, std::vector<uint8_t> &out) {
    for (;;) {
        int s = decode(b, lit);
        if (s < 0) return "bad literal/length code";
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return "";
        } else {
            s -= 257;
            if (s >= 29) return "bad length symbol";
            const int len = kLenBase[s] + b.need(kLenExtra[s]);
            const int ds = decode(b, dist);
            if (ds < 0 || ds >= 30) return "bad distance code";
            const size_t d = (size_t)kDistBase[ds] + b.need(kDistExtra[ds]);
            if (b.bad) return "truncated stream";
            if (d > out.size()) return "distance beyond output";
            const size_t from = out.size() - d;
            for (int k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

std::string inflate_raw(Bits &b, std::vector<uint8_t> &out) {
    for (;;) {
        const int last = b.need(1);
        const int type = b.need(2);
        if (b.bad) return "truncated stream";
        if (type == 0) {
            b.align(); // stored block: LEN and NLEN start at the next byte boundary
            const unsigned len = (unsigned)b.need(16), nlen = (unsigned)b.need(16);
            if (b.bad || (len ^ 0xFFFFu) != nlen) return "bad stored block";
            for (unsigned k = 0; k < len; k++) {
                const int v = b.need(8);
                if (b.bad) return "truncated stored block";
                out.push_back((uint8_t)v);
            }
        } else if (type == 1) {
            static const FixedCodes fixed;
            const std::string e = codes(b, fixed.lit, fixed.dist, out);
            if (!e.empty()) return e;
        } else if (type == 2) {
            const int nlen = b.need(5) + 257, ndist = b.need(5) + 1, ncode = b.need(4) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            int lengths[320] = {};
            for (int k = 0; k < ncode; k++) lengths[order[k]] = b.need(3);
            Huff cl;
            if (b.bad || !build(cl, lengths, 19)) return "bad code-length code";
            int k = 0;
            std::memset(lengths, 0, sizeof lengths);
            while (k < nlen + ndist) {
                const int s = decode(b, cl);
                if (s < 0) return "bad code length";
                if (s < 16) {
                    lengths[k++] = s;
                } else {
                    int rep, val = 0;
                    if (s == 16) {
                        if (k == 0) return "repeat without a previous length";
                        val = lengths[k - 1];
                        rep = 3 + b.need(2);
                    } else if (s == 17) {
                        rep = 3 + b.need(3);
                    } else {
                        rep = 11 + b.need(7);
                    }
                    if (k + rep > nlen + ndist) return "too many code lengths";
                    while (rep--) lengths[k++] = val;
                }
            }
            Huff lit, dist;
            if (!build(lit, lengths, nlen) || !build(dist, lengths + nlen, ndist)) return "bad dynamic codes";
            const std::string e = codes(b, lit, dist, out);
            if (!e.empty()) return e;
        } else {
            return "bad block type";
        }
        if (last) return "";
    }
}

// ---------------------------------------------------------------- checksums
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t k = 0; k < 256; k++) {
            uint32_t v = k;
            for (int j = 0; j < 8; j++) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            t[k] = v;
        }
    }
};

uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0) {
    static const CrcTable table; // built once, thread-safe static initialisation
    c = ~c;
    for (size_t i = 0; i < n; i++) c = table.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return ~c;
}

uint32_t adler32(const uint8_t *p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; i++) {
        a = (a + p[i]) % 65521;
        b = (b + a) % 65521;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
void put32(std::vector<uint8_t> &v, uint32_t x) {
    for (int s = 24; s >= 0; s -= 8) v.push_back((uint8_t)(x >> s));
}

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

} // namespace

std::string zlib_inflate(const uint8_t *data, size_t n, std::vector<uint8_t> &out) {
    if (n < 6) return "zlib stream too short";
    if ((data[0] & 0x0F) != 8 || ((data[0] << 8) | data[1]) % 31 != 0 || (data[1] & 0x20))
        return "unsupported zlib header";
    Bits b{data + 2, n - 2};
    std::string e = inflate_raw(b, out);
    if (!e.empty()) return e;
    const size_t end = b.byte_end(); // the remaining bits of the last byte are padding
    if (end + 4 > b.n) return "missing adler32";
    if (be32(b.p + end) != adler32(out.data(), out.size())) return "adler32 mismatch";
    return "";
}

std::vector<uint8_t> zlib_store(const uint8_t *data, size_t n) {
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        const size_t len = n - off > 65535 ? 65535 : n - off;
        z.push_back(off + len == n ? 1 : 0);
        z.push_back((uint8_t)(len & 0xFF));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xFF));
        z.push_back((uint8_t)((~len >> 8) & 0xFF));
        z.insert(z.end(), data + off, data + off + len);
        off += len;
    } while (off < n);
    put32(z, adler32(data, n));
    return z;
}

std::string read_png(const std::string &path, Image &img) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return "cannot open " + path;
    std::vector<uint8_t> file;
    uint8_t chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) file.insert(file.end(), chunk, chunk + got);
    std::fclose(f);
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (file.size() < 8 || std::memcmp(file.data(), sig, 8)) return path + ": not a PNG file";
    size_t pos = 8;
    int w = 0, h = 0, depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat;
    while (pos + 12 <= file.size()) {
        const uint32_t len = be32(&file[pos]);
        if (pos + 12 + (size_t)len > file.size()) return path + ": truncated chunk";
        const uint8_t *type = &file[pos + 4], *dat = &file[pos + 8];
        if (crc32(type, len + 4) != be32(dat + len)) return path + ": chunk CRC mismatch";
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = (int)be32(dat);
            h = (int)be32(dat + 4);
            depth = dat[8];
            ctype = dat[9];
            interlace = dat[12];
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), dat, dat + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (w <= 0 || h <= 0) return path + ": missing IHDR";
    if (depth != 8 || interlace || (ctype != 0 && ctype != 2 && ctype != 4 && ctype != 6))
        return path + ": only 8-bit non-interlaced gray, gray+alpha, RGB or RGBA PNGs are supported";
    const int spp = ctype == 0 ? 1 : (ctype == 4 ? 2 : (ctype == 2 ? 3 : 4));
    std::vector<uint8_t> raw;
    std::string e = zlib_inflate(idat.data(), idat.size(), raw);
    if (!e.empty()) return path + ": " + e;
    const size_t stride = (size_t)w * spp;
    if (raw.size() < (stride + 1) * h) return path + ": image data too short";
    std::vector<uint8_t> cur(stride), prev(stride, 0);
    img.width = w;
    img.height = h;
    img.channels = (ctype == 0 || ctype == 4) ? 1 : 3;
    img.pixels.assign((size_t)w * h * img.channels, 0);
    for (int y = 0; y < h; y++) {
        const uint8_t ft = raw[y * (stride + 1)];
        const uint8_t *src = &raw[y * (stride + 1) + 1];
        for (size_t x = 0; x < stride; x++) {
            const int a = x >= (size_t)spp ? cur[x - spp] : 0, b = prev[x], c = x >= (size_t)spp ? prev[x - spp] : 0;
            int v = src[x];
            switch (ft) {
            case 0: break;
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) >> 1; break;
            case 4: v += paeth(a, b, c); break;
            default: return path + ": bad filter type";
            }
            cur[x] = (uint8_t)v;
        }
        uint8_t *dst = &img.pixels[(size_t)y * w * img.channels];
        for (int x = 0; x < w; x++) {
            if (img.channels == 1) {
                dst[x] = cur[(size_t)x * spp];
            } else { // RGB(A) -> B, G, R
                dst[3 * x] = cur[(size_t)x * spp + 2];
                dst[3 * x + 1] = cur[(size_t)x * spp + 1];
                dst[3 * x + 2] = cur[(size_t)x * spp];
            }
        }
        std::swap(cur, prev);
    }
    return "";
}

std::string write_png_gray(const std::string &path, int w, int h, int depth, const void *pixels) {
    if (depth != 8 && depth != 16) return "bit depth must be 8 or 16";
    const size_t row = (size_t)w * (depth / 8);
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * h);
    for (int y = 0; y < h; y++) {
        raw.push_back(0);
        if (depth == 8) {
            const uint8_t *p = static_cast<const uint8_t *>(pixels) + (size_t)y * w;
            raw.insert(raw.end(), p, p + w);
        } else {
            const uint16_t *p = static_cast<const uint16_t *>(pixels) + (size_t)y * w;
            for (int x = 0; x < w; x++) {
                raw.push_back((uint8_t)(p[x] >> 8));
                raw.push_back((uint8_t)(p[x] & 0xFF));
            }
        }
    }
    std::vector<uint8_t> png = {137, 80, 78, 71, 13, 10, 26, 10};
    auto chunk = [&](const char *type, const std::vector<uint8_t> &data) {
        put32(png, (uint32_t)data.size());
        const size_t start = png.size();
        png.insert(png.end(), type, type + 4);
        png.insert(png.end(), data.begin(), data.end());
        put32(png, crc32(&png[start], data.size() + 4));
    };
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.push_back((uint8_t)depth);
    ihdr.push_back(0); // gray
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    chunk("IHDR", ihdr);
    chunk("IDAT", zlib_store(raw.data(), raw.size()));
    chunk("IEND", {});
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return "cannot write " + path;
    const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
    std::fclose(f);
    return ok ? "" : "short write to " + path;
}

} // namespace pngio
