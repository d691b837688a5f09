// Host-side JPEG decoder for scene ingestion: Texture::load (Imaging.h:44-79)
// reads textures through stb_image, and many of the reference's scenes use
// JPEG albedo maps.  Written from ITU-T T.81 (Huffman-coded baseline,
// extended 8-bit and progressive processes; Annexes B, C, F.2, G.2) and JFIF
// 1.02 (YCbCr -> RGB): inverse DCT in double precision, chroma upsampled with
// the triangle filter (weights 3/4, 1/4 per axis, as JFIF readers commonly
// do), samples rounded to nearest.  stb_image uses fixed-point arithmetic for
// the same steps, so samples agree with it to within a few levels rather than
// bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pgx.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// Position in the 8x8 block (row-major) of the k-th coefficient in zig-zag order (T.81 Figure A.6).
constexpr uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JpegError {
    std::string what;
};
[[noreturn]] void fail(const char* what) { throw JpegError{what}; }

// Canonical Huffman table (T.81 Annex C), decoded with a 9-bit lookahead and
// the MINCODE / MAXCODE / VALPTR procedure of F.2.2.3 for longer codes.
struct Huffman {
    bool present = false;
    uint8_t values[256] = {};
    int32_t mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
    uint8_t fast_len[512] = {};  // 0: not decodable from 9 bits
    uint8_t fast_val[512] = {};

    void build(const uint8_t* counts, const uint8_t* vals, int nvals) {
        std::memcpy(values, vals, (size_t)nvals);
        std::memset(fast_len, 0, sizeof(fast_len));
        int code = 0, k = 0;
        for (int len = 1; len <= 16; len++) {
            valptr[len] = k;
            mincode[len] = code;
            for (int i = 0; i < counts[len - 1]; i++, k++, code++) {
                if (code >= (1 << len)) fail("invalid Huffman table");  // over-subscribed lengths
                if (len <= 9) {
                    const int shift = 9 - len;
                    for (int f = code << shift; f < ((code + 1) << shift); f++) {
                        fast_len[f] = (uint8_t)len;
                        fast_val[f] = values[k];
                    }
                }
            }
            maxcode[len] = counts[len - 1] ? code - 1 : -1;
            if (code > (1 << len)) fail("invalid Huffman table");
            code <<= 1;
        }
        maxcode[17] = 0x7fffffff;
        present = true;
    }
};

// Entropy-coded segment reader: byte stuffing (0xFF00) removed, a marker
// stops the data and zeros are fed after it (T.81 F.1.2.3, B.1.1.5).
struct BitReader {
    const uint8_t* p;
    const uint8_t* end;
    uint64_t acc = 0;
    int nbits = 0;
    bool at_marker = false;

    void fill() {
        while (nbits <= 56) {
            uint8_t b = 0;
            if (!at_marker && p < end) {
                b = *p;
                if (b == 0xFF) {
                    const uint8_t nx = (p + 1 < end) ? p[1] : 0xD9;
                    if (nx == 0x00) {
                        p += 2;
                    } else {
                        at_marker = true;  // leave the marker for the parser
                        b = 0;
                    }
                } else {
                    p++;
                }
            }
            acc |= (uint64_t)b << (56 - nbits);
            nbits += 8;
        }
    }
    int bits(int n) {
        if (n == 0) return 0;
        if (nbits < n) fill();
        const int v = (int)(acc >> (64 - n));
        acc <<= n;
        nbits -= n;
        return v;
    }
    int bit() { return bits(1); }
    // F.2.2.1 EXTEND of an n-bit magnitude category
    int receive_extend(int n) {
        if (n == 0) return 0;
        if (n > 16) fail("invalid coefficient size");
        const int v = bits(n);
        return v < (1 << (n - 1)) ? v - (1 << n) + 1 : v;
    }
    int decode(const Huffman& h) {
        if (!h.present) fail("scan uses an undefined Huffman table");
        if (nbits < 16) fill();
        const int look = (int)(acc >> 55);
        const int fl = h.fast_len[look];
        if (fl) {
            acc <<= fl;
            nbits -= fl;
            return h.fast_val[look];
        }
        int code = 0;
        for (int len = 1; len <= 16; len++) {
            code = (code << 1) | bit();
            if (code <= h.maxcode[len]) return h.values[h.valptr[len] + code - h.mincode[len]];
        }
        fail("invalid Huffman code");
    }
    // Restart: drop the bits left in the byte and step over the RSTn marker.
    void restart(int expect) {
        acc = 0;
        nbits = 0;
        at_marker = false;
        if (p + 1 < end && p[0] == 0xFF && p[1] == 0xD0 + (expect & 7)) {
            p += 2;
        } else {
            // tolerate a missing marker: resynchronise on the next RSTn if any
            while (p + 1 < end && !(p[0] == 0xFF && p[1] >= 0xD0 && p[1] <= 0xD7)) p++;
            if (p + 1 < end) p += 2;
        }
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int bw = 0, bh = 0;        // blocks covering the component's samples
    int pbw = 0, pbh = 0;      // blocks allocated (a whole number of MCUs)
    std::vector<int16_t> coef;  // pbw * pbh blocks of 64, natural order
    int dc_pred = 0;
    int td = 0, ta = 0;
    std::vector<uint8_t> plane;  // pbw*8 x pbh*8 samples after the IDCT
};

struct Decoder {
    const uint8_t* data;
    const uint8_t* end;
    uint16_t qt[4][64] = {};  // natural order
    bool qt_present[4] = {};
    Huffman dc[4], ac[4];
    std::vector<Component> comp;
    int width = 0, height = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool progressive = false, frame_seen = false;
    int restart_interval = 0;
    int adobe_transform = -1;
    bool jfif = false;

    int u16(const uint8_t* q) const { return (q[0] << 8) | q[1]; }

    void read_dqt(const uint8_t* q, int len) {
        const uint8_t* e = q + len;
        while (q < e) {
            const int pq = q[0] >> 4, tq = q[0] & 15;
            if (tq > 3 || pq > 1) fail("invalid quantisation table");
            q++;
            if (q + 64 * (pq + 1) > e) fail("truncated quantisation table");
            for (int k = 0; k < 64; k++) qt[tq][kZigzag[k]] = pq ? (uint16_t)u16(q + 2 * k) : q[k];
            qt_present[tq] = true;
            q += 64 * (pq + 1);
        }
    }
    void read_dht(const uint8_t* q, int len) {
        const uint8_t* e = q + len;
        while (q < e) {
            if (q + 17 > e) fail("truncated Huffman table");
            const int tc = q[0] >> 4, th = q[0] & 15;
            if (tc > 1 || th > 3) fail("invalid Huffman table id");
            int n = 0;
            for (int i = 0; i < 16; i++) n += q[1 + i];
            if (n > 256 || q + 17 + n > e) fail("invalid Huffman table size");
            (tc ? ac[th] : dc[th]).build(q + 1, q + 17, n);
            q += 17 + n;
        }
    }
    void read_sof(const uint8_t* q, int len, int marker) {
        if (frame_seen) fail("more than one frame");
        if (len < 6) fail("truncated frame header");
        if (q[0] != 8) fail("only 8-bit samples are supported");
        height = u16(q + 1);
        width = u16(q + 3);
        const int nc = q[5];
        if (width <= 0 || height <= 0) fail("image without a size (DNL) is not supported");
        if ((nc != 1 && nc != 3) || len < 6 + 3 * nc) fail("only 1- and 3-component images are supported");
        progressive = marker == 0xC2;
        comp.resize(nc);
        for (int i = 0; i < nc; i++) {
            Component& c = comp[i];
            c.id = q[6 + 3 * i];
            c.h = q[7 + 3 * i] >> 4;
            c.v = q[7 + 3 * i] & 15;
            c.tq = q[8 + 3 * i];
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) fail("invalid component parameters");
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        if ((int64_t)mcux * mcuy * hmax * vmax * nc > (int64_t)1 << 23) fail("image too large");
        for (Component& c : comp) {
            c.bw = ((width * c.h + hmax - 1) / hmax + 7) / 8;
            c.bh = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            c.pbw = mcux * c.h;
            c.pbh = mcuy * c.v;
            c.coef.assign((size_t)c.pbw * c.pbh * 64, 0);
        }
        frame_seen = true;
    }

    // One block of a sequential scan (F.2.2).
    void block_sequential(BitReader& br, Component& c, int16_t* blk) {
        const int t = br.decode(dc[c.td]);
        if (t > 11) fail("invalid DC difference");
        c.dc_pred += br.receive_extend(t);
        blk[0] = (int16_t)c.dc_pred;
        for (int k = 1; k < 64;) {
            const int rs = br.decode(ac[c.ta]);
            const int r = rs >> 4, s = rs & 15;
            if (s) {
                k += r;
                if (k > 63) fail("coefficient index out of range");
                blk[kZigzag[k]] = (int16_t)br.receive_extend(s);
                k++;
            } else if (r == 15) {
                k += 16;
            } else {
                break;
            }
        }
    }

    // Progressive scans (G.2): DC first / refinement, AC first / refinement.
    void block_dc_first(BitReader& br, Component& c, int16_t* blk, int al) {
        const int t = br.decode(dc[c.td]);
        if (t > 11) fail("invalid DC difference");
        c.dc_pred += br.receive_extend(t);
        blk[0] = (int16_t)(c.dc_pred * (1 << al));
    }
    void block_dc_refine(BitReader& br, int16_t* blk, int al) {
        if (br.bit()) blk[0] = (int16_t)(blk[0] | (1 << al));
    }
    void block_ac_first(BitReader& br, Component& c, int16_t* blk, int ss, int se, int al, int& eobrun) {
        if (eobrun > 0) {
            eobrun--;
            return;
        }
        for (int k = ss; k <= se; k++) {
            const int rs = br.decode(ac[c.ta]);
            const int r = rs >> 4, s = rs & 15;
            if (s) {
                k += r;
                if (k > 63) fail("coefficient index out of range");
                blk[kZigzag[k]] = (int16_t)(br.receive_extend(s) * (1 << al));
            } else if (r == 15) {
                k += 15;
            } else {
                eobrun = (1 << r) - 1;
                if (r) eobrun += br.bits(r);
                break;
            }
        }
    }
    void refine_nonzero(BitReader& br, int16_t& co, int p1) {
        if (br.bit() && (co & p1) == 0) co = (int16_t)(co >= 0 ? co + p1 : co - p1);
    }
    void block_ac_refine(BitReader& br, Component& c, int16_t* blk, int ss, int se, int al, int& eobrun) {
        const int p1 = 1 << al;
        int k = ss;
        if (eobrun <= 0) {
            for (; k <= se; k++) {
                const int rs = br.decode(ac[c.ta]);
                int r = rs >> 4;
                const int s = rs & 15;
                int val = 0;
                if (s) {
                    if (s != 1) fail("invalid refinement coefficient");
                    val = br.bit() ? p1 : -p1;
                } else if (r != 15) {
                    eobrun = 1 << r;
                    if (r) eobrun += br.bits(r);
                    break;  // the rest of the band is refined below
                }
                // Step over coefficients already nonzero (each takes a correction
                // bit) and r zero ones; a new coefficient goes at the next zero.
                for (; k <= se; k++) {
                    int16_t& co = blk[kZigzag[k]];
                    if (co != 0) {
                        refine_nonzero(br, co, p1);
                    } else {
                        if (r == 0) {
                            if (val) co = (int16_t)val;
                            break;
                        }
                        r--;
                    }
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; k++) {
                int16_t& co = blk[kZigzag[k]];
                if (co != 0) refine_nonzero(br, co, p1);
            }
            eobrun--;
        }
    }

    // One scan (B.2.3): returns the position after its entropy-coded data.
    const uint8_t* scan(const uint8_t* q, int len, const uint8_t* seg_end) {
        if (!frame_seen) fail("scan before frame header");
        if (len < 1) fail("invalid scan header");
        const int ns = q[0];
        if (ns < 1 || ns > 4 || len < 4 + 2 * ns) fail("invalid scan header");
        std::vector<Component*> sc;
        for (int i = 0; i < ns; i++) {
            const int id = q[1 + 2 * i];
            Component* c = nullptr;
            for (Component& cc : comp)
                if (cc.id == id) c = &cc;
            if (!c) fail("scan names an unknown component");
            c->td = q[2 + 2 * i] >> 4;
            c->ta = q[2 + 2 * i] & 15;
            if (c->td > 3 || c->ta > 3) fail("invalid table selector");
            sc.push_back(c);
        }
        const int ss = q[1 + 2 * ns], se = q[2 + 2 * ns], ah = q[3 + 2 * ns] >> 4, al = q[3 + 2 * ns] & 15;
        if (progressive) {
            if (ss > se || se > 63 || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13)
                fail("invalid progressive scan parameters");
        } else if (ss != 0 || se != 63 || ah != 0 || al != 0) {
            fail("invalid sequential scan parameters");
        }
        for (Component* c : sc) c->dc_pred = 0;
        BitReader br{seg_end, end};
        int eobrun = 0, rst = 0, todo = restart_interval;

        auto decode_block = [&](Component& c, int bx, int by) {
            int16_t* blk = c.coef.data() + ((size_t)by * c.pbw + bx) * 64;
            if (!progressive)
                block_sequential(br, c, blk);
            else if (ss == 0)
                ah == 0 ? block_dc_first(br, c, blk, al) : block_dc_refine(br, blk, al);
            else
                ah == 0 ? block_ac_first(br, c, blk, ss, se, al, eobrun) : block_ac_refine(br, c, blk, ss, se, al, eobrun);
        };
        auto restart_point = [&]() {
            if (restart_interval && --todo == 0) {
                br.restart(rst++);
                todo = restart_interval;
                eobrun = 0;
                for (Component* c : sc) c->dc_pred = 0;
            }
        };

        if (ns == 1) {
            // non-interleaved: the component's own blocks in raster order (A.2.2)
            Component& c = *sc[0];
            for (int by = 0; by < c.bh; by++)
                for (int bx = 0; bx < c.bw; bx++) {
                    decode_block(c, bx, by);
                    restart_point();
                }
        } else {
            for (int my = 0; my < mcuy; my++)
                for (int mx = 0; mx < mcux; mx++) {
                    for (Component* c : sc)
                        for (int y = 0; y < c->v; y++)
                            for (int x = 0; x < c->h; x++) decode_block(*c, mx * c->h + x, my * c->v + y);
                    restart_point();
                }
        }
        // the data ends at the next marker that is not RSTn
        const uint8_t* p = br.p;
        while (p + 1 < end && !(p[0] == 0xFF && p[1] != 0x00 && !(p[1] >= 0xD0 && p[1] <= 0xD7))) p++;
        return p;
    }

    // Dequantisation and 8x8 inverse DCT (A.3.3) of every block.
    void reconstruct() {
        double cosv[8][8];  // cosv[x][u] = C(u)/2 cos((2x+1) u pi / 16)
        for (int x = 0; x < 8; x++)
            for (int u = 0; u < 8; u++)
                cosv[x][u] = (u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * kPi / 16.0);
        for (Component& c : comp) {
            if (!qt_present[c.tq]) fail("component uses an undefined quantisation table");
            const uint16_t* q = qt[c.tq];
            const int stride = c.pbw * 8;
            c.plane.assign((size_t)stride * c.pbh * 8, 0);
            for (int by = 0; by < c.pbh; by++)
                for (int bx = 0; bx < c.pbw; bx++) {
                    const int16_t* blk = c.coef.data() + ((size_t)by * c.pbw + bx) * 64;
                    double f[64], tmp[64];
                    bool ac = false, row_nz[8] = {};
                    for (int i = 0; i < 64; i++) {
                        f[i] = (double)blk[i] * q[i];
                        if (blk[i]) {
                            row_nz[i >> 3] = true;
                            if (i) ac = true;
                        }
                    }
                    uint8_t* out = c.plane.data() + (size_t)by * 8 * stride + bx * 8;
                    if (!ac) {
                        const double s = f[0] * cosv[0][0] * cosv[0][0] + 128.0;
                        const uint8_t v = (uint8_t)std::min(255.0, std::max(0.0, std::floor(s + 0.5)));
                        for (int y = 0; y < 8; y++) std::memset(out + (size_t)y * stride, v, 8);
                        continue;
                    }
                    // rows: f(v, u) -> tmp(v, x); rows of zero coefficients stay zero
                    for (int v = 0; v < 8; v++) {
                        if (!row_nz[v]) continue;
                        for (int x = 0; x < 8; x++) {
                            double s = 0.0;
                            for (int u = 0; u < 8; u++) s += cosv[x][u] * f[v * 8 + u];
                            tmp[v * 8 + x] = s;
                        }
                    }
                    for (int y = 0; y < 8; y++)
                        for (int x = 0; x < 8; x++) {
                            double s = 0.0;
                            for (int v = 0; v < 8; v++)
                                if (row_nz[v]) s += cosv[y][v] * tmp[v * 8 + x];
                            s += 128.0;
                            out[(size_t)y * stride + x] = (uint8_t)std::min(255.0, std::max(0.0, std::floor(s + 0.5)));
                        }
                }
        }
    }

    // Component sample at full resolution: triangle filter for 2x factors,
    // replication otherwise.
    int sample(const Component& c, int x, int y) const {
        const int stride = c.pbw * 8;
        const int cw = c.pbw * 8, ch = c.pbh * 8;
        const int fx = hmax / c.h, fy = vmax / c.v;
        const bool tx = fx == 2 && hmax % c.h == 0, ty = fy == 2 && vmax % c.v == 0;
        if (!tx && !ty) {
            const int sx = std::min(x * c.h / hmax, cw - 1), sy = std::min(y * c.v / vmax, ch - 1);
            return c.plane[(size_t)sy * stride + sx];
        }
        // the component's own samples (the rest of its blocks is padding)
        const int cwa = std::min(cw, (width * c.h + hmax - 1) / hmax), cha = std::min(ch, (height * c.v + vmax - 1) / vmax);
        const int sx0 = std::min(tx ? x >> 1 : x * c.h / hmax, cwa - 1);
        const int sy0 = std::min(ty ? y >> 1 : y * c.v / vmax, cha - 1);
        const int sx1 = tx ? std::min(std::max(sx0 + ((x & 1) ? 1 : -1), 0), cwa - 1) : sx0;
        const int sy1 = ty ? std::min(std::max(sy0 + ((y & 1) ? 1 : -1), 0), cha - 1) : sy0;
        const int a = c.plane[(size_t)sy0 * stride + sx0], b = c.plane[(size_t)sy0 * stride + sx1];
        const int d = c.plane[(size_t)sy1 * stride + sx0], e = c.plane[(size_t)sy1 * stride + sx1];
        if (tx && ty) return (9 * a + 3 * b + 3 * d + e + 8) >> 4;
        if (tx) return (3 * a + b + 2) >> 2;
        return (3 * a + d + 2) >> 2;
    }

    void output(uint8_t* out) const {
        const int nc = (int)comp.size();
        if (nc == 1) {
            const Component& c = comp[0];
            for (int y = 0; y < height; y++)
                for (int x = 0; x < width; x++) out[(size_t)y * width + x] = (uint8_t)sample(c, x, y);
            return;
        }
        // RGB-coded data: an Adobe marker with transform 0, or components named R, G, B
        const bool rgb = adobe_transform == 0 ||
                         (!jfif && adobe_transform < 0 && comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B');
        const bool full = comp[0].h == hmax && comp[0].v == vmax && comp[1].h == hmax && comp[1].v == vmax &&
                          comp[2].h == hmax && comp[2].v == vmax;
        for (int y = 0; y < height; y++)
            for (int x = 0; x < width; x++) {
                int Y, cb, cr;
                if (full) {  // every component at full resolution: no resampling
                    const size_t i = (size_t)y * comp[0].pbw * 8 + x;
                    Y = comp[0].plane[i];
                    cb = comp[1].plane[(size_t)y * comp[1].pbw * 8 + x];
                    cr = comp[2].plane[(size_t)y * comp[2].pbw * 8 + x];
                } else {
                    Y = sample(comp[0], x, y);
                    cb = sample(comp[1], x, y);
                    cr = sample(comp[2], x, y);
                }
                uint8_t* o = out + ((size_t)y * width + x) * 3;
                if (rgb) {
                    o[0] = (uint8_t)Y;
                    o[1] = (uint8_t)cb;
                    o[2] = (uint8_t)cr;
                    continue;
                }
                const double r = Y + 1.402 * (cr - 128);
                const double g = Y - 0.344136 * (cb - 128) - 0.714136 * (cr - 128);
                const double b = Y + 1.772 * (cb - 128);
                auto to8 = [](double v) { return (uint8_t)std::min(255.0, std::max(0.0, std::floor(v + 0.5))); };
                o[0] = to8(r);
                o[1] = to8(g);
                o[2] = to8(b);
            }
    }

    // Parses the marker segments; with decode, also the scans.
    void run(bool decode) {
        const uint8_t* p = data;
        if (end - p < 4 || p[0] != 0xFF || p[1] != 0xD8) fail("not a JPEG file (no SOI marker)");
        p += 2;
        bool scans = false;
        while (p < end) {
            if (p[0] != 0xFF) {
                p++;  // tolerate junk between segments
                continue;
            }
            if (p + 1 >= end) break;
            const int m = p[1];
            if (m == 0xFF) {  // fill byte before a marker (B.1.1.2)
                p++;
                continue;
            }
            p += 2;
            if (m == 0x01 || (m >= 0xD0 && m <= 0xD7)) continue;
            if (m == 0xD9) break;  // EOI
            if (p + 2 > end) fail("truncated marker segment");
            const int len = u16(p);
            if (len < 2 || p + len > end) fail("truncated marker segment");
            const uint8_t* q = p + 2;
            const int n = len - 2;
            switch (m) {
                case 0xC0:
                case 0xC1:
                case 0xC2:
                    read_sof(q, n, m);
                    if (!decode) return;
                    break;
                case 0xC3:
                case 0xC5:
                case 0xC6:
                case 0xC7:
                case 0xC9:
                case 0xCA:
                case 0xCB:
                case 0xCD:
                case 0xCE:
                case 0xCF:
                    fail("lossless, hierarchical and arithmetic-coded JPEG are not supported");
                case 0xC4:
                    read_dht(q, n);
                    break;
                case 0xDB:
                    read_dqt(q, n);
                    break;
                case 0xDD:
                    if (n < 2) fail("invalid restart interval");
                    restart_interval = u16(q);
                    break;
                case 0xE0:
                    if (n >= 5 && std::memcmp(q, "JFIF\0", 5) == 0) jfif = true;
                    break;
                case 0xEE:
                    if (n >= 12 && std::memcmp(q, "Adobe", 5) == 0) adobe_transform = q[11];
                    break;
                case 0xDA: {
                    p = scan(q, n, p + len);
                    scans = true;
                    continue;
                }
                default:
                    break;  // APPn, COM and others carry nothing the decoder needs
            }
            p += len;
        }
        if (!frame_seen) fail("no frame header");
        if (decode && !scans) fail("no scan");
    }
};

int set_msg(char* msg, int32_t msg_size, const std::string& text) {
    if (msg && msg_size > 0) {
        std::snprintf(msg, (size_t)msg_size, "%s", text.c_str());
    }
    return PGX_ERR_INVALID_ARG;
}

}  // namespace

extern "C" int pgx_image_decode_jpeg(const uint8_t* data, int64_t size, int32_t* width, int32_t* height,
                                     int32_t* channels, uint8_t* out, int64_t out_size, char* msg, int32_t msg_size) {
    if (!data || size <= 0 || !width || !height || !channels) return set_msg(msg, msg_size, "null argument");
    try {
        Decoder d;
        d.data = data;
        d.end = data + size;
        d.run(out != nullptr);
        *width = d.width;
        *height = d.height;
        *channels = (int32_t)d.comp.size();
        if (!out) return PGX_OK;
        const int64_t need = (int64_t)d.width * d.height * (int64_t)d.comp.size();
        if (out_size < need) return set_msg(msg, msg_size, "output buffer too small");
        d.reconstruct();
        d.output(out);
        return PGX_OK;
    } catch (const JpegError& e) {
        return set_msg(msg, msg_size, e.what);
    } catch (const std::bad_alloc&) {
        return set_msg(msg, msg_size, "out of memory");
    }
}
