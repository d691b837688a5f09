// Scene files in the reference's format, read on the host in C++:
// `loadScene` (SceneLoader.h:222-269) with `loadInstance`
// (SceneLoader.h:104-220), `GEMScene::load` (GEMLoader.h:853-882) and
// `GEMModelLoader::load` (GEMLoader.h:430-457), `Texture::load`
// (Imaging.h:44-79).  The result feeds pgx_scene_upload with the triangles,
// materials, textures, environment and camera the reference builds.
//
// Rules kept from the reference (and from its JSON reader): top-level keys
// and instance keys are visited in sorted order (std::map, last duplicate
// wins); numbers are kept as std::stof of their text and turned back into
// strings with std::to_string; booleans become "1"/"0"; numeric properties
// are read with std::stof / std::stoi semantics (a leading valid prefix,
// defaults when nothing converts); vectors split on single spaces.  Each
// instance gets one material; vertices are transformed in float32 in the
// reference's operation order (Matrix::mulPoint; normals by the transposed
// MESA inverse, then normalised); triangles of zero area are dropped; index
// offsets between the meshes of one file are counted in indices, as the
// reference counts them.  Textures are decoded here: 8-bit PNG (zlib
// inflate per RFC 1950/1951, written for this file), Radiance HDR, 24/32-bit
// BMP and TGA, and JPEG through pgx_image_decode_jpeg; a file that cannot be
// read becomes the 1x1 white default, as a failing stbi_load does there.
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pgx_ctx.h"

namespace {

struct LoadError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

[[noreturn]] void failf(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw LoadError(buf);
}

bool read_file(const std::string& path, std::vector<uint8_t>& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
    bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
uint32_t le32(const uint8_t* p) { return (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0]; }
uint16_t le16(const uint8_t* p) { return (uint16_t)(p[0] | p[1] << 8); }

// ---- inflate (RFC 1951) --------------------------------------------------------------

class Inflater {
  public:
    Inflater(const uint8_t* p, size_t n) : p_(p), n_(n) {}

    void run(std::vector<uint8_t>& out) {
        int final = 0;
        while (!final) {
            final = bits(1);
            int type = bits(2);
            if (type == 0) {
                stored(out);
            } else if (type == 1) {
                Huff lit, dist;
                fixed(lit, dist);
                block(out, lit, dist);
            } else if (type == 2) {
                Huff lit, dist;
                dynamic(lit, dist);
                block(out, lit, dist);
            } else {
                failf("inflate: invalid block type");
            }
        }
    }

  private:
    // Canonical Huffman code: number of codes of each length and the
    // symbols in code order; decoded one bit at a time.
    struct Huff {
        uint16_t count[16] = {};
        std::vector<uint16_t> symbol;
    };

    const uint8_t* p_;
    size_t n_;
    size_t pos_ = 0;
    uint32_t bitbuf_ = 0;
    int bitcnt_ = 0;

    int bits(int need) {
        uint32_t v = bitbuf_;
        while (bitcnt_ < need) {
            if (pos_ >= n_) failf("inflate: data ends early");
            v |= (uint32_t)p_[pos_++] << bitcnt_;
            bitcnt_ += 8;
        }
        bitbuf_ = v >> need;
        bitcnt_ -= need;
        return (int)(v & ((1u << need) - 1u));
    }

    static void make(Huff& h, const uint8_t* lengths, int n) {
        for (int i = 0; i < 16; i++) h.count[i] = 0;
        for (int s = 0; s < n; s++) h.count[lengths[s]]++;
        h.count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= h.count[len];
            if (left < 0) failf("inflate: over-subscribed code");
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++) offs[len + 1] = (uint16_t)(offs[len] + h.count[len]);
        h.symbol.assign((size_t)n, 0);
        for (int s = 0; s < n; s++)
            if (lengths[s]) h.symbol[offs[lengths[s]]++] = (uint16_t)s;
    }

    int decode(const Huff& h) {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= bits(1);
            int cnt = h.count[len];
            if (code - cnt < first) return h.symbol[(size_t)(index + (code - first))];
            index += cnt;
            first += cnt;
            first <<= 1;
            code <<= 1;
        }
        failf("inflate: invalid code");
    }

    void stored(std::vector<uint8_t>& out) {
        bitbuf_ = 0;
        bitcnt_ = 0;
        if (pos_ + 4 > n_) failf("inflate: data ends early");
        unsigned len = p_[pos_] | p_[pos_ + 1] << 8;
        unsigned nlen = p_[pos_ + 2] | p_[pos_ + 3] << 8;
        pos_ += 4;
        if (len != (~nlen & 0xFFFFu)) failf("inflate: stored block length mismatch");
        if (pos_ + len > n_) failf("inflate: data ends early");
        out.insert(out.end(), p_ + pos_, p_ + pos_ + len);
        pos_ += len;
    }

    static void fixed(Huff& lit, Huff& dist) {
        uint8_t l[288];
        for (int s = 0; s < 144; s++) l[s] = 8;
        for (int s = 144; s < 256; s++) l[s] = 9;
        for (int s = 256; s < 280; s++) l[s] = 7;
        for (int s = 280; s < 288; s++) l[s] = 8;
        make(lit, l, 288);
        uint8_t d[30];
        for (int s = 0; s < 30; s++) d[s] = 5;
        make(dist, d, 30);
    }

    void dynamic(Huff& lit, Huff& dist) {
        static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        int nlen = bits(5) + 257, ndist = bits(5) + 1, ncode = bits(4) + 4;
        if (nlen > 286 || ndist > 30) failf("inflate: bad code counts");
        uint8_t lengths[320] = {};
        for (int i = 0; i < ncode; i++) lengths[order[i]] = (uint8_t)bits(3);
        Huff lencode;
        make(lencode, lengths, 19);
        int idx = 0;
        while (idx < nlen + ndist) {
            int sym = decode(lencode);
            if (sym < 16) {
                lengths[idx++] = (uint8_t)sym;
                continue;
            }
            int rep;
            uint8_t val = 0;
            if (sym == 16) {
                if (idx == 0) failf("inflate: repeat with no previous length");
                val = lengths[idx - 1];
                rep = 3 + bits(2);
            } else if (sym == 17) {
                rep = 3 + bits(3);
            } else {
                rep = 11 + bits(7);
            }
            if (idx + rep > nlen + ndist) failf("inflate: too many lengths");
            while (rep--) lengths[idx++] = val;
        }
        if (lengths[256] == 0) failf("inflate: no end-of-block code");
        make(lit, lengths, nlen);
        make(dist, lengths + nlen, ndist);
    }

    void block(std::vector<uint8_t>& out, const Huff& lit, const Huff& dist) {
        static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                           31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
        static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
        static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
        static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
        for (;;) {
            int sym = decode(lit);
            if (sym < 256) {
                out.push_back((uint8_t)sym);
            } else if (sym == 256) {
                return;
            } else {
                sym -= 257;
                if (sym >= 29) failf("inflate: invalid length symbol");
                int len = lbase[sym] + bits(lext[sym]);
                int ds = decode(dist);
                if (ds >= 30) failf("inflate: invalid distance symbol");
                size_t d = (size_t)dbase[ds] + (size_t)bits(dext[ds]);
                if (d > out.size()) failf("inflate: distance too far back");
                size_t from = out.size() - d;
                for (int k = 0; k < len; k++) out.push_back(out[from + (size_t)k]);
            }
            if (out.size() > ((size_t)1 << 31)) failf("inflate: output too large");
        }
    }
};

// ---- images ---------------------------------------------------------------------------

struct Image8 {
    int w = 0, h = 0, c = 0;
    std::vector<uint8_t> px;  // h * w * c, rows top-down
};

// 8-bit, non-interlaced PNG (colour types 0, 2, 3, 4, 6); palettes expand to RGB.
Image8 read_png(const std::vector<uint8_t>& d) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0) failf("not a PNG file");
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int bitd = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette;
    while (pos + 8 <= d.size()) {
        uint32_t len = be32(&d[pos]);
        const uint8_t* tag = &d[pos + 4];
        if (pos + 12 + (size_t)len > d.size()) failf("PNG chunk runs past the end");
        const uint8_t* body = &d[pos + 8];
        pos += 12 + (size_t)len;
        if (!std::memcmp(tag, "IHDR", 4) && len >= 13) {
            w = be32(body);
            h = be32(body + 4);
            bitd = body[8];
            ctype = body[9];
            interlace = body[12];
        } else if (!std::memcmp(tag, "PLTE", 4)) {
            palette.assign(body, body + len);
        } else if (!std::memcmp(tag, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(tag, "IEND", 4)) {
            break;
        }
    }
    if (bitd != 8 || interlace != 0) failf("only 8-bit non-interlaced PNGs are supported");
    int ch;
    switch (ctype) {
        case 0: ch = 1; break;
        case 2: ch = 3; break;
        case 3: ch = 1; break;
        case 4: ch = 2; break;
        case 6: ch = 4; break;
        default: failf("unknown PNG colour type");
    }
    if (w == 0 || h == 0 || (uint64_t)w * h * (uint64_t)ch > ((uint64_t)1 << 30)) failf("bad PNG size");
    if (idat.size() < 2) failf("PNG without image data");
    if ((idat[0] & 15) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0) failf("bad zlib header");
    std::vector<uint8_t> raw;
    Inflater(idat.data() + 2, idat.size() - 2).run(raw);
    const size_t stride = (size_t)w * ch;
    if (raw.size() < (stride + 1) * h) failf("PNG image data too short");
    Image8 img;
    img.w = (int)w;
    img.h = (int)h;
    img.c = ch;
    img.px.assign(stride * h, 0);
    std::vector<int> prev(stride, 0), cur(stride, 0);
    size_t p = 0;
    for (uint32_t y = 0; y < h; y++) {
        int ft = raw[p];
        const uint8_t* line = &raw[p + 1];
        p += 1 + stride;
        for (size_t x = 0; x < stride; x++) {
            int a = x >= (size_t)ch ? cur[x - ch] : 0;
            int b = prev[x];
            int c = x >= (size_t)ch ? prev[x - ch] : 0;
            int pr;
            switch (ft) {
                case 0: pr = 0; break;
                case 1: pr = a; break;
                case 2: pr = b; break;
                case 3: pr = (a + b) >> 1; break;
                case 4: {
                    int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
                    pr = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: failf("bad PNG filter type");
            }
            cur[x] = (line[x] + pr) & 255;
        }
        for (size_t x = 0; x < stride; x++) img.px[y * stride + x] = (uint8_t)cur[x];
        std::swap(prev, cur);
    }
    if (ctype == 3) {
        Image8 rgb;
        rgb.w = img.w;
        rgb.h = img.h;
        rgb.c = 3;
        rgb.px.resize((size_t)img.w * img.h * 3);
        for (size_t i = 0; i < (size_t)img.w * img.h; i++) {
            size_t k = (size_t)img.px[i] * 3;
            if (k + 3 > palette.size()) failf("PNG palette index out of range");
            for (int j = 0; j < 3; j++) rgb.px[3 * i + j] = palette[k + j];
        }
        return rgb;
    }
    return img;
}

// Uncompressed 24/32-bit BMP, rows top-down, RGB(A).
Image8 read_bmp(const std::vector<uint8_t>& d) {
    if (d.size() < 54 || d[0] != 'B' || d[1] != 'M') failf("not a BMP file");
    uint32_t off = le32(&d[10]);
    int32_t w = (int32_t)le32(&d[18]), h = (int32_t)le32(&d[22]);
    int bpp = le16(&d[28]);
    uint32_t comp = le32(&d[30]);
    if ((comp != 0 && comp != 3) || (bpp != 24 && bpp != 32)) failf("only uncompressed 24/32-bit BMPs are supported");
    if (w <= 0 || h == 0 || h == INT32_MIN) failf("bad BMP size");
    const int ch = bpp / 8;
    const int ah = h < 0 ? -h : h;
    const size_t stride = ((size_t)w * ch + 3) & ~(size_t)3;
    if ((size_t)off + stride * ah > d.size()) failf("BMP data too short");
    Image8 img;
    img.w = w;
    img.h = ah;
    img.c = ch;
    img.px.resize((size_t)w * ah * ch);
    for (int y = 0; y < ah; y++) {
        const uint8_t* row = &d[off + stride * (size_t)(h > 0 ? ah - 1 - y : y)];
        for (int x = 0; x < w; x++) {
            uint8_t* o = &img.px[((size_t)y * w + x) * ch];
            o[0] = row[x * ch + 2];
            o[1] = row[x * ch + 1];
            o[2] = row[x * ch + 0];
            if (ch == 4) o[3] = row[x * ch + 3];
        }
    }
    return img;
}

// True-colour TGA (types 2 and 10, 24/32-bit), rows top-down, RGB(A).
Image8 read_tga(const std::vector<uint8_t>& d) {
    if (d.size() < 18) failf("not a TGA file");
    int idlen = d[0], cmtype = d[1], itype = d[2];
    int w = le16(&d[12]), h = le16(&d[14]), bpp = d[16], desc = d[17];
    if (cmtype != 0 || (itype != 2 && itype != 10) || (bpp != 24 && bpp != 32))
        failf("only true-colour 24/32-bit TGAs are supported");
    if (w == 0 || h == 0) failf("bad TGA size");
    const int ch = bpp / 8;
    size_t pos = 18 + (size_t)idlen;
    const size_t n = (size_t)w * h;
    std::vector<uint8_t> px(n * ch);
    if (itype == 2) {
        if (pos + n * ch > d.size()) failf("TGA data too short");
        std::memcpy(px.data(), &d[pos], n * ch);
    } else {
        size_t i = 0;
        while (i < n) {
            if (pos >= d.size()) failf("TGA data too short");
            int hdr = d[pos++];
            size_t cnt = (size_t)(hdr & 127) + 1;
            if (i + cnt > n) failf("TGA run past the image");
            if (hdr & 128) {
                if (pos + ch > d.size()) failf("TGA data too short");
                for (size_t k = 0; k < cnt; k++) std::memcpy(&px[(i + k) * ch], &d[pos], (size_t)ch);
                pos += (size_t)ch;
            } else {
                if (pos + cnt * ch > d.size()) failf("TGA data too short");
                std::memcpy(&px[i * ch], &d[pos], cnt * ch);
                pos += cnt * ch;
            }
            i += cnt;
        }
    }
    Image8 img;
    img.w = w;
    img.h = h;
    img.c = ch;
    img.px.resize(n * ch);
    for (int y = 0; y < h; y++) {
        int sy = (desc & 0x20) ? y : h - 1 - y;
        for (int x = 0; x < w; x++) {
            const uint8_t* s = &px[((size_t)sy * w + x) * ch];
            uint8_t* o = &img.px[((size_t)y * w + x) * ch];
            o[0] = s[2];
            o[1] = s[1];
            o[2] = s[0];
            if (ch == 4) o[3] = s[3];
        }
    }
    return img;
}

Image8 read_jpeg(const std::vector<uint8_t>& d) {
    int32_t w = 0, h = 0, c = 0;
    char msg[256] = {0};
    if (pgx_image_decode_jpeg(d.data(), (int64_t)d.size(), &w, &h, &c, nullptr, 0, msg, sizeof(msg)) != PGX_OK)
        failf("%s", msg);
    Image8 img;
    img.w = w;
    img.h = h;
    img.c = c;
    img.px.resize((size_t)w * h * c);
    if (pgx_image_decode_jpeg(d.data(), (int64_t)d.size(), &w, &h, &c, img.px.data(), (int64_t)img.px.size(), msg,
                              sizeof(msg)) != PGX_OK)
        failf("%s", msg);
    return img;
}

struct TexF {
    int w = 1, h = 1;
    std::vector<float> rgb{1.f, 1.f, 1.f};  // Texture::loadDefault (Imaging.h:36-42)
};

// Radiance RGBE: texel = byte * 2^(e - 136) (0 when e == 0).  Widths
// 8..32767 start every scanline with a run-length header (2, 2, width); a
// scanline without one switches to flat pixels from that point of the file on.
TexF read_hdr(const std::vector<uint8_t>& d) {
    auto starts = [&](const char* s) { return d.size() >= std::strlen(s) && !std::memcmp(d.data(), s, std::strlen(s)); };
    if (!starts("#?RADIANCE\n") && !starts("#?RGBE\n")) failf("not a Radiance file");
    size_t pos = 0;
    auto line = [&]() {
        size_t e = pos;
        while (e < d.size() && d[e] != '\n') e++;
        if (e >= d.size()) failf("Radiance header ends early");
        std::string s((const char*)&d[pos], e - pos);
        pos = e + 1;
        return s;
    };
    while (!line().empty()) {
    }
    std::string res = line();
    char a[8] = {0}, b[8] = {0};
    int h = 0, w = 0;
    if (std::sscanf(res.c_str(), "%7s %d %7s %d", a, &h, b, &w) != 4 || std::strcmp(a, "-Y") || std::strcmp(b, "+X"))
        failf("unsupported Radiance orientation");
    if (w <= 0 || h <= 0 || (int64_t)w * h > ((int64_t)1 << 28)) failf("bad Radiance size");
    std::vector<uint8_t> rgbe((size_t)w * h * 4, 0);
    bool flat = !(w >= 8 && w < 32768);
    if (!flat) {
        for (int y = 0; y < h && !flat; y++) {
            if (pos + 4 > d.size()) failf("Radiance data too short");
            if (!(d[pos] == 2 && d[pos + 1] == 2 && d[pos + 2] < 128)) {
                flat = true;
                break;
            }
            if ((d[pos + 2] << 8 | d[pos + 3]) != w) failf("invalid decoded scanline length");
            pos += 4;
            for (int c = 0; c < 4; c++) {
                int x = 0;
                while (x < w) {
                    if (pos >= d.size()) failf("Radiance data too short");
                    int cnt = d[pos++];
                    if (cnt > 128) {
                        cnt -= 128;
                        if (x + cnt > w || pos >= d.size()) failf("bad Radiance run");
                        for (int k = 0; k < cnt; k++) rgbe[((size_t)y * w + x + k) * 4 + c] = d[pos];
                        pos++;
                    } else {
                        if (cnt == 0 || x + cnt > w || pos + cnt > d.size()) failf("bad Radiance run");
                        for (int k = 0; k < cnt; k++) rgbe[((size_t)y * w + x + k) * 4 + c] = d[pos + k];
                        pos += (size_t)cnt;
                    }
                    x += cnt;
                }
            }
        }
    }
    if (flat) {
        if (pos + rgbe.size() > d.size()) failf("Radiance data too short");
        std::memcpy(rgbe.data(), &d[pos], rgbe.size());
    }
    TexF t;
    t.w = w;
    t.h = h;
    t.rgb.resize((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; i++) {
        int e = rgbe[4 * i + 3];
        float f = e == 0 ? 0.f : (float)std::ldexp(1.0, e - 136);
        for (int c = 0; c < 3; c++) t.rgb[3 * i + c] = (float)rgbe[4 * i + c] * f;
    }
    return t;
}

bool ends_with_ci(const std::string& s, const char* suf) {
    size_t n = std::strlen(suf);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; i++) {
        char c = s[s.size() - n + i];
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
        if (c != suf[i]) return false;
    }
    return true;
}

// Texture::load: RGB float texels; 8-bit images scaled by 1/255 with texel i
// read from bytes [i*C, i*C+3) whatever the channel count C (bytes past the
// end read as 0).
TexF load_texture(const std::string& path) {
    std::vector<uint8_t> d;
    if (path.find(".hdr") != std::string::npos) {
        try {
            if (!read_file(path, d)) return TexF();
            return read_hdr(d);
        } catch (const LoadError&) {
            return TexF();
        }
    }
    Image8 img;
    try {
        const bool png = ends_with_ci(path, ".png"), bmp = ends_with_ci(path, ".bmp"), tga = ends_with_ci(path, ".tga");
        const bool jpg = ends_with_ci(path, ".jpg") || ends_with_ci(path, ".jpeg");
        if (!(png || bmp || tga || jpg)) return TexF();
        if (!read_file(path, d)) return TexF();
        img = png ? read_png(d) : bmp ? read_bmp(d) : tga ? read_tga(d) : read_jpeg(d);
    } catch (const LoadError&) {
        return TexF();
    }
    TexF t;
    t.w = img.w;
    t.h = img.h;
    const size_t n = (size_t)img.w * img.h;
    t.rgb.resize(n * 3);
    const float inv = 1.0f / 255.0f;
    for (size_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            size_t k = i * (size_t)img.c + (size_t)c;
            t.rgb[3 * i + c] = (float)(k < img.px.size() ? img.px[k] : 0) * inv;
        }
    return t;
}

// ---- scene.json ---------------------------------------------------------------------

struct Json {
    enum Type { NUL, BOOL, NUM, STR, ARR, OBJ } type = NUL;
    bool b = false;
    float num = 0.f;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    // std::to_string of booleans and numbers, strings as they are, else "".
    std::string as_str() const {
        char buf[64];
        switch (type) {
            case BOOL: return b ? "1" : "0";
            case NUM: std::snprintf(buf, sizeof(buf), "%f", (double)num); return buf;
            case STR: return str;
            default: return "";
        }
    }
};

// std::stof: strtof on the longest valid prefix; false where stof throws.
bool stof_prefix(const std::string& s, float& out) {
    errno = 0;
    char* end = nullptr;
    float v = std::strtof(s.c_str(), &end);
    if (end == s.c_str() || errno != 0) return false;
    out = v;
    return true;
}

// std::stoi: leading decimal integer after optional whitespace and sign.
bool stoi_prefix(const std::string& s, int& out) {
    size_t i = 0;
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\v' || s[i] == '\f' || s[i] == '\r')) i++;
    size_t j = i;
    if (j < s.size() && (s[j] == '+' || s[j] == '-')) j++;
    size_t k = j;
    while (k < s.size() && s[k] >= '0' && s[k] <= '9') k++;
    if (k == j) return false;
    errno = 0;
    long long v = std::strtoll(s.substr(i, k - i).c_str(), nullptr, 10);
    if (errno != 0 || v < INT32_MIN || v > INT32_MAX) return false;
    out = (int)v;
    return true;
}

class JsonParser {
  public:
    explicit JsonParser(const std::string& s) : s_(s) {}
    Json parse() {
        Json v = value();
        ws();
        if (i_ != s_.size()) failf("scene.json: trailing data at %zu", i_);
        return v;
    }

  private:
    const std::string& s_;
    size_t i_ = 0;
    int depth_ = 0;

    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) i_++;
    }
    bool lit(const char* w) {
        size_t n = std::strlen(w);
        if (s_.compare(i_, n, w) == 0) {
            i_ += n;
            return true;
        }
        return false;
    }
    static void utf8(std::string& o, unsigned cp) {
        if (cp < 0x80) {
            o += (char)cp;
        } else if (cp < 0x800) {
            o += (char)(0xC0 | (cp >> 6));
            o += (char)(0x80 | (cp & 63));
        } else if (cp < 0x10000) {
            o += (char)(0xE0 | (cp >> 12));
            o += (char)(0x80 | ((cp >> 6) & 63));
            o += (char)(0x80 | (cp & 63));
        } else {
            o += (char)(0xF0 | (cp >> 18));
            o += (char)(0x80 | ((cp >> 12) & 63));
            o += (char)(0x80 | ((cp >> 6) & 63));
            o += (char)(0x80 | (cp & 63));
        }
    }
    unsigned hex4() {
        if (i_ + 4 > s_.size()) failf("scene.json: bad escape");
        unsigned v = 0;
        for (int k = 0; k < 4; k++) {
            char c = s_[i_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else failf("scene.json: bad escape");
        }
        return v;
    }
    std::string string() {
        std::string o;
        i_++;  // opening quote
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c != '\\') {
                o += c;
                continue;
            }
            if (i_ >= s_.size()) break;
            char e = s_[i_++];
            switch (e) {
                case 'n': o += '\n'; break;
                case 't': o += '\t'; break;
                case 'r': o += '\r'; break;
                case 'b': o += '\b'; break;
                case 'f': o += '\f'; break;
                case 'u': {
                    unsigned cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00 && s_.compare(i_, 2, "\\u") == 0) {
                        i_ += 2;
                        unsigned lo = hex4();
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(o, cp);
                    break;
                }
                default: o += e; break;
            }
        }
        if (i_ >= s_.size()) failf("scene.json: unterminated string");
        i_++;
        return o;
    }
    Json value() {
        if (++depth_ > 64) failf("scene.json: nested too deeply");
        ws();
        if (i_ >= s_.size()) failf("scene.json: unexpected end");
        Json v;
        char c = s_[i_];
        if (c == '{') {
            v.type = Json::OBJ;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == '}') {
                i_++;
            } else {
                for (;;) {
                    ws();
                    if (i_ >= s_.size() || s_[i_] != '"') failf("scene.json: expected a key at %zu", i_);
                    std::string k = string();
                    ws();
                    if (i_ >= s_.size() || s_[i_] != ':') failf("scene.json: expected ':' at %zu", i_);
                    i_++;
                    v.obj[k] = value();  // last duplicate wins
                    ws();
                    if (i_ < s_.size() && s_[i_] == ',') {
                        i_++;
                        continue;
                    }
                    if (i_ < s_.size() && s_[i_] == '}') {
                        i_++;
                        break;
                    }
                    failf("scene.json: expected ',' or '}' at %zu", i_);
                }
            }
        } else if (c == '[') {
            v.type = Json::ARR;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == ']') {
                i_++;
            } else {
                for (;;) {
                    v.arr.push_back(value());
                    ws();
                    if (i_ < s_.size() && s_[i_] == ',') {
                        i_++;
                        continue;
                    }
                    if (i_ < s_.size() && s_[i_] == ']') {
                        i_++;
                        break;
                    }
                    failf("scene.json: expected ',' or ']' at %zu", i_);
                }
            }
        } else if (c == '"') {
            v.type = Json::STR;
            v.str = string();
        } else if (lit("true")) {
            v.type = Json::BOOL;
            v.b = true;
        } else if (lit("false")) {
            v.type = Json::BOOL;
        } else if (lit("null")) {
            v.type = Json::NUL;
        } else {
            size_t j = i_;
            if (j < s_.size() && s_[j] == '-') j++;
            while (j < s_.size() && ((s_[j] >= '0' && s_[j] <= '9') || s_[j] == '.' || s_[j] == 'e' || s_[j] == 'E' ||
                                     s_[j] == '+' || s_[j] == '-'))
                j++;
            if (j == i_) failf("scene.json: unexpected character at %zu", i_);
            std::string tok = s_.substr(i_, j - i_);
            i_ = j;
            v.type = Json::NUM;
            if (!stof_prefix(tok, v.num)) failf("scene.json: number out of float range: %s", tok.c_str());
        }
        depth_--;
        return v;
    }
};

float prop_float(const std::map<std::string, std::string>& p, const char* k, float def) {
    auto it = p.find(k);
    if (it == p.end() || it->second.empty()) return def;
    float v;
    return stof_prefix(it->second, v) ? v : def;
}

int prop_int(const std::map<std::string, std::string>& p, const char* k, int def) {
    auto it = p.find(k);
    if (it == p.end() || it->second.empty()) return def;
    int v;
    return stoi_prefix(it->second, v) ? v : def;
}

// Words split on single spaces (no word after a trailing separator), each
// through stof; empty or unparsable words and missing entries are 0.
void prop_vec3(const std::map<std::string, std::string>& p, const char* k, float out[3]) {
    out[0] = out[1] = out[2] = 0.f;
    auto it = p.find(k);
    if (it == p.end()) return;
    const std::string& s = it->second;
    std::vector<std::string> words;
    size_t start = 0;
    while (start < s.size()) {
        size_t e = s.find(' ', start);
        if (e == std::string::npos) {
            words.push_back(s.substr(start));
            break;
        }
        words.push_back(s.substr(start, e - start));
        start = e + 1;
    }
    for (size_t i = 0; i < words.size() && i < 3; i++) {
        float v;
        if (!words[i].empty() && stof_prefix(words[i], v)) out[i] = v;
    }
}

// ---- GEM meshes ------------------------------------------------------------------------

struct GemMesh {
    std::vector<float> verts;  // V x 11: position, normal, tangent, u, v
    std::vector<uint32_t> idx;
};

std::vector<GemMesh> read_gem(const std::string& path) {
    std::vector<uint8_t> d;
    if (!read_file(path, d)) failf("%s: cannot read the mesh file", path.c_str());
    size_t pos = 0;
    auto u32 = [&]() {
        if (pos + 4 > d.size()) failf("%s: mesh file ends early", path.c_str());
        uint32_t v = le32(&d[pos]);
        pos += 4;
        return v;
    };
    if (u32() != 4058972161u) failf("%s is not a GE Model File", path.c_str());
    if (u32() != 0) failf("%s: animated meshes are not supported", path.c_str());
    uint32_t nmesh = u32();
    std::vector<GemMesh> out;
    for (uint32_t m = 0; m < nmesh; m++) {
        uint32_t nprop = u32();
        for (uint32_t k = 0; k < 2 * nprop; k++) {
            uint32_t len = u32();
            if (pos + len > d.size()) failf("%s: mesh file ends early", path.c_str());
            pos += len;
        }
        GemMesh g;
        uint32_t nv = u32();
        if (pos + (size_t)nv * 44 > d.size()) failf("%s: mesh file ends early", path.c_str());
        g.verts.resize((size_t)nv * 11);
        std::memcpy(g.verts.data(), &d[pos], (size_t)nv * 44);
        pos += (size_t)nv * 44;
        uint32_t ni = u32();
        if (pos + (size_t)ni * 4 > d.size()) failf("%s: mesh file ends early", path.c_str());
        g.idx.resize(ni);
        std::memcpy(g.idx.data(), &d[pos], (size_t)ni * 4);
        pos += (size_t)ni * 4;
        out.push_back(std::move(g));
    }
    return out;
}

// ---- float32 matrix helpers in the reference's operation order ---------------------------

// Matrix::invert (MyMath.h:286-323): cofactors, determinant, scale.
void invert16(const float* m, float* out) {
    auto t = [&](int a, int b, int c) { return m[a] * m[b] * m[c]; };
    float inv[16];
    inv[0] = t(5, 10, 15) - t(5, 11, 14) - t(9, 6, 15) + t(9, 7, 14) + t(13, 6, 11) - t(13, 7, 10);
    inv[4] = -m[4] * m[10] * m[15] + t(4, 11, 14) + t(8, 6, 15) - t(8, 7, 14) - t(12, 6, 11) + t(12, 7, 10);
    inv[8] = t(4, 9, 15) - t(4, 11, 13) - t(8, 5, 15) + t(8, 7, 13) + t(12, 5, 11) - t(12, 7, 9);
    inv[12] = -m[4] * m[9] * m[14] + t(4, 10, 13) + t(8, 5, 14) - t(8, 6, 13) - t(12, 5, 10) + t(12, 6, 9);
    inv[1] = -m[1] * m[10] * m[15] + t(1, 11, 14) + t(9, 2, 15) - t(9, 3, 14) - t(13, 2, 11) + t(13, 3, 10);
    inv[5] = t(0, 10, 15) - t(0, 11, 14) - t(8, 2, 15) + t(8, 3, 14) + t(12, 2, 11) - t(12, 3, 10);
    inv[9] = -m[0] * m[9] * m[15] + t(0, 11, 13) + t(8, 1, 15) - t(8, 3, 13) - t(12, 1, 11) + t(12, 3, 9);
    inv[13] = t(0, 9, 14) - t(0, 10, 13) - t(8, 1, 14) + t(8, 2, 13) + t(12, 1, 10) - t(12, 2, 9);
    inv[2] = t(1, 6, 15) - t(1, 7, 14) - t(5, 2, 15) + t(5, 3, 14) + t(13, 2, 7) - t(13, 3, 6);
    inv[6] = -m[0] * m[6] * m[15] + t(0, 7, 14) + t(4, 2, 15) - t(4, 3, 14) - t(12, 2, 7) + t(12, 3, 6);
    inv[10] = t(0, 5, 15) - t(0, 7, 13) - t(4, 1, 15) + t(4, 3, 13) + t(12, 1, 7) - t(12, 3, 5);
    inv[14] = -m[0] * m[5] * m[14] + t(0, 6, 13) + t(4, 1, 14) - t(4, 2, 13) - t(12, 1, 6) + t(12, 2, 5);
    inv[3] = -m[1] * m[6] * m[11] + t(1, 7, 10) + t(5, 2, 11) - t(5, 3, 10) - t(9, 2, 7) + t(9, 3, 6);
    inv[7] = t(0, 6, 11) - t(0, 7, 10) - t(4, 2, 11) + t(4, 3, 10) + t(8, 2, 7) - t(8, 3, 6);
    inv[11] = -m[0] * m[5] * m[11] + t(0, 7, 9) + t(4, 1, 11) - t(4, 3, 9) - t(8, 1, 7) + t(8, 3, 5);
    inv[15] = t(0, 5, 10) - t(0, 6, 9) - t(4, 1, 10) + t(4, 2, 9) + t(8, 1, 6) - t(8, 2, 5);
    float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0.f) det = 1.f;
    det = 1.f / det;
    for (int i = 0; i < 16; i++) out[i] = inv[i] * det;
}

struct LoadedScene {
    std::vector<pgx_triangle> tris;
    std::vector<pgx_material> mats;
    std::vector<TexF> textures;
    bool has_env = false;
    TexF env;
    pgx_camera camera{};
};

// The BSDF loadInstance makes for one instance (SceneLoader.h:107-176);
// false when `bsdf` names no known BSDF (the instance is skipped).
bool instance_material(const std::map<std::string, std::string>& keys, pgx_material& m,
                       const std::function<int(const std::string&)>& texture) {
    static const std::map<std::string, int> names = {
        {"diffuse", PGX_BSDF_DIFFUSE}, {"orennayar", PGX_BSDF_ORENNAYAR}, {"glass", PGX_BSDF_GLASS},
        {"mirror", PGX_BSDF_MIRROR},   {"plastic", PGX_BSDF_PLASTIC},     {"dielectric", PGX_BSDF_DIELECTRIC},
        {"conductor", PGX_BSDF_CONDUCTOR}};
    auto b = keys.find("bsdf");
    auto k = names.find(b == keys.end() ? std::string() : b->second);
    if (k == names.end()) return false;
    int kind = k->second;
    m = pgx_material{};
    auto refl = keys.find("reflectance");
    m.albedo_texture = texture(refl == keys.end() ? std::string() : refl->second);
    if (kind == PGX_BSDF_ORENNAYAR) m.sigma = prop_float(keys, "alpha", 1.0f);
    if (kind == PGX_BSDF_GLASS || kind == PGX_BSDF_PLASTIC || kind == PGX_BSDF_DIELECTRIC) {
        m.int_ior = prop_float(keys, "intIOR", 1.33f);
        m.ext_ior = prop_float(keys, "extIOR", 1.0f);
    }
    if (kind == PGX_BSDF_PLASTIC || kind == PGX_BSDF_DIELECTRIC || kind == PGX_BSDF_CONDUCTOR)
        m.roughness = prop_float(keys, "roughness", 1.0f);
    if (kind == PGX_BSDF_DIELECTRIC && m.roughness < 0.001f) {  // SceneLoader.h:145-149
        kind = PGX_BSDF_GLASS;
        m.roughness = 0.f;
    }
    if (kind == PGX_BSDF_CONDUCTOR) {
        prop_vec3(keys, "eta", m.eta);
        prop_vec3(keys, "k", m.k);
    }
    m.kind = kind;
    auto em = keys.find("emission");
    if (em != keys.end() && !em->second.empty()) prop_vec3(keys, "emission", m.emission);
    if (prop_int(keys, "coatingThickness", 0) > 0) {
        // LayeredBSDF (Materials.h:855-897) forwards every query to its base
        // and is made after addLight: the wrapped material emits nothing.
        m.layered = 1;
        m.emission[0] = m.emission[1] = m.emission[2] = 0.f;
    }
    return true;
}

void load(const std::string& dir_in, LoadedScene& out) {
    std::string d = dir_in;
    while (d.size() > 1 && d.back() == '/') d.pop_back();
    std::vector<uint8_t> raw;
    if (!read_file(d + "/scene.json", raw)) failf("%s/scene.json: cannot read", d.c_str());
    std::string text(raw.begin(), raw.end());
    Json js = JsonParser(text).parse();
    if (js.type != Json::OBJ) failf("scene.json: top level is not an object");
    std::map<std::string, std::string> props;
    std::vector<const Json*> instances;
    for (const auto& kv : js.obj) {
        if (kv.second.type != Json::ARR) {
            props[kv.first] = kv.second.as_str();
        } else {
            for (const Json& inst : kv.second.arr) instances.push_back(&inst);
        }
    }
    pgx_camera& cam = out.camera;
    prop_vec3(props, "from", cam.from);
    prop_vec3(props, "to", cam.to);
    prop_vec3(props, "up", cam.up);
    cam.fov_degrees = prop_float(props, "fov", 45.0f);
    cam.width = prop_int(props, "width", 1920);
    cam.height = prop_int(props, "height", 1080);
    cam.flip_x = prop_int(props, "flipX", 0) == 1 ? 1 : 0;

    std::map<std::string, int> tex_ids;
    auto texture = [&](const std::string& name) {
        const std::string key = d + "/" + name;
        auto it = tex_ids.find(key);
        if (it != tex_ids.end()) return it->second;
        int id = (int)out.textures.size();
        tex_ids[key] = id;
        out.textures.push_back(load_texture(key));
        return id;
    };

    for (const Json* inst : instances) {
        if (inst->type != Json::OBJ) continue;
        std::map<std::string, std::string> keys;
        for (const auto& kv : inst->obj)
            if (kv.first != "filename" && kv.first != "world") keys[kv.first] = kv.second.as_str();
        auto fn = inst->obj.find("filename");
        std::string mesh_file = fn == inst->obj.end() ? std::string() : fn->second.as_str();
        std::vector<GemMesh> meshes = read_gem(d + "/" + mesh_file);
        pgx_material m;
        if (!instance_material(keys, m, texture)) continue;  // "Error in loading" (SceneLoader.h:177-181)
        const uint32_t mat_index = (uint32_t)out.mats.size();
        out.mats.push_back(m);
        float world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        auto w = inst->obj.find("world");
        if (w != inst->obj.end() && w->second.type == Json::ARR)
            for (int i = 0; i < 16; i++)
                world[i] = (i < (int)w->second.arr.size() && w->second.arr[(size_t)i].type == Json::NUM)
                               ? w->second.arr[(size_t)i].num
                               : 0.f;
        float inv[16], vt[16];
        invert16(world, inv);
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) vt[r * 4 + c] = inv[c * 4 + r];
        std::vector<float> verts;
        std::vector<int64_t> ind;
        for (const GemMesh& g : meshes) {
            const int64_t off = (int64_t)ind.size();  // counted in indices, as the reference does
            for (uint32_t i : g.idx) ind.push_back((int64_t)i + off);
            verts.insert(verts.end(), g.verts.begin(), g.verts.end());
        }
        if (verts.empty()) continue;
        const int64_t nv = (int64_t)(verts.size() / 11);
        std::vector<float> P((size_t)nv * 3), N((size_t)nv * 3);
        for (int64_t i = 0; i < nv; i++) {
            const float* v = &verts[(size_t)i * 11];
            float x = v[0], y = v[1], z = v[2];
            P[3 * i] = ((x * world[0] + y * world[1]) + z * world[2]) + world[3];
            P[3 * i + 1] = ((x * world[4] + y * world[5]) + z * world[6]) + world[7];
            P[3 * i + 2] = ((x * world[8] + y * world[9]) + z * world[10]) + world[11];
            float nx = v[3], ny = v[4], nz = v[5];
            float a = (nx * vt[0] + ny * vt[1]) + nz * vt[2];
            float b = (nx * vt[4] + ny * vt[5]) + nz * vt[6];
            float c = (nx * vt[8] + ny * vt[9]) + nz * vt[10];
            float l = std::sqrt((a * a + b * b) + c * c);
            float il = 1.f / l;
            N[3 * i] = a * il;
            N[3 * i + 1] = b * il;
            N[3 * i + 2] = c * il;
        }
        for (size_t t = 0; t + 3 <= ind.size(); t += 3) {
            pgx_triangle tr{};
            for (int k = 0; k < 3; k++) {
                const int64_t vi = ind[t + (size_t)k];
                if (vi < 0 || vi >= nv) failf("%s: vertex index %lld out of range", mesh_file.c_str(), (long long)vi);
                for (int j = 0; j < 3; j++) {
                    tr.v[k].p[j] = P[(size_t)vi * 3 + j];
                    tr.v[k].n[j] = N[(size_t)vi * 3 + j];
                }
                tr.v[k].u = verts[(size_t)vi * 11 + 9];
                tr.v[k].v = verts[(size_t)vi * 11 + 10];
            }
            tr.material = mat_index;
            // Triangle::init's area (Geometry.h:86-92); zero-area triangles are dropped.
            const float* p0 = tr.v[0].p;
            const float* p1 = tr.v[1].p;
            const float* p2 = tr.v[2].p;
            float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
            float e2[3] = {p0[0] - p2[0], p0[1] - p2[1], p0[2] - p2[2]};
            float cx = e1[1] * e2[2] - e1[2] * e2[1];
            float cy = e1[2] * e2[0] - e1[0] * e2[2];
            float cz = e1[0] * e2[1] - e1[1] * e2[0];
            float area = std::sqrt((cx * cx + cy * cy) + cz * cz) * 0.5f;
            if (area > 0.f) out.tris.push_back(tr);
        }
    }
    auto env = props.find("envmap");
    if (env != props.end() && !env->second.empty()) {
        out.has_env = true;
        out.env = load_texture(d + "/" + env->second);
    }
}

// Owner of a pgx_scene_data's arrays.
struct SceneData {
    pgx_scene_data pub{};
    LoadedScene s;
    std::vector<pgx_texture> tex;
};

}  // namespace

extern "C" int pgx_scene_read(const char* dir, pgx_scene_data** out, char* msg, int32_t msg_size) {
    if (msg && msg_size > 0) msg[0] = 0;
    if (!dir || !out) {
        if (msg && msg_size > 0) std::snprintf(msg, (size_t)msg_size, "pgx_scene_read: null argument");
        return PGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    std::unique_ptr<SceneData> sd(new SceneData());
    try {
        load(dir, sd->s);
    } catch (const std::exception& e) {
        if (msg && msg_size > 0) std::snprintf(msg, (size_t)msg_size, "%s", e.what());
        return PGX_ERR_INVALID_ARG;
    }
    for (const TexF& t : sd->s.textures) sd->tex.push_back(pgx_texture{t.w, t.h, t.rgb.data()});
    pgx_scene_data& p = sd->pub;
    p.triangles = sd->s.tris.data();
    p.ntris = (int64_t)sd->s.tris.size();
    p.materials = sd->s.mats.data();
    p.nmats = (int32_t)sd->s.mats.size();
    p.textures = sd->tex.data();
    p.ntextures = (int32_t)sd->tex.size();
    p.has_env = sd->s.has_env ? 1 : 0;
    p.env = sd->s.has_env ? pgx_texture{sd->s.env.w, sd->s.env.h, sd->s.env.rgb.data()} : pgx_texture{0, 0, nullptr};
    p.camera = sd->s.camera;
    p.internal = sd.get();
    *out = &sd.release()->pub;
    return PGX_OK;
}

extern "C" void pgx_scene_data_free(pgx_scene_data* d) {
    if (d) delete static_cast<SceneData*>(d->internal);
}

extern "C" int pgx_scene_load(pgx_ctx* ctx, const char* dir) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    pgx_scene_data* d = nullptr;
    char msg[512];
    int rc = pgx_scene_read(dir, &d, msg, sizeof(msg));
    if (rc != PGX_OK) return pgx_fail(ctx, rc, "pgx_scene_load: %s", msg);
    rc = pgx_scene_upload(ctx, d->triangles, d->ntris, d->materials, d->nmats, d->ntextures ? d->textures : nullptr,
                          d->ntextures, d->has_env ? &d->env : nullptr, &d->camera);
    pgx_scene_data_free(d);
    return rc;
}
