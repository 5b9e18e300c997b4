// GROMACS .xtc trajectories: a decoder and an encoder of the published compressed-coordinate
// format, written for this project (the reference links libxdrfile: read_xtc_natoms,
// read_xtc_n_frames, xdr_seek and read_xtc, calcIR.cu:212-223, 341-395).
//
// A frame is XDR (big-endian, 4-byte units): magic 1995, natoms, step, time (float), the
// 3 x 3 box (floats), natoms again, then the coordinates.  Up to 9 atoms they are plain
// floats.  Otherwise: precision p, the minimum and maximum integer coordinate per axis,
// the starting small-difference index, a byte count and that many bytes (padded to 4) of
// a bit stream.  Coordinates are integers round(x p) (half away from zero).  The stream
// holds, per "large" atom, its three coordinates relative to the minima as one mixed-radix
// integer (or per-axis fields when an axis spans more than 2^24), a flag bit, optionally a
// 5-bit run code (run length in atoms x 3, plus the change of the small index), and then
// the run's "small" atoms as mixed-radix triples of differences offset by half the current
// small range.  The first small atom of a run precedes the large atom in the output (the
// format swaps them, which favours water: oxygen small relative to a hydrogen), later ones
// follow in order, each relative to the previously emitted atom.  A flag of 0 repeats the
// previous run length.  The table of small ranges (about 2^(i/3) for index i) and the bit
// counts are part of the format and are reproduced as specified.
#include "cir_internal.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

constexpr int XTC_MAGIC = 1995;
constexpr int FIRSTIDX = 9;
// smallest range index with a nonzero range; index i: triples of values below RANGE[i] fit
// in i bits
constexpr unsigned RANGE[] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 8, 10, 12, 16, 20, 25, 32, 40, 50, 64, 80, 101, 128, 161, 203, 256,
    322, 406, 512, 645, 812, 1024, 1290, 1625, 2048, 2580, 3250, 4096, 5060, 6501, 8192, 10321, 13003,
    16384, 20642, 26007, 32768, 41285, 52015, 65536, 82570, 104031, 131072, 165140, 208063, 262144, 330280,
    416127, 524287, 660561, 832255, 1048576, 1321122, 1664510, 2097152, 2642245, 3329021, 4194304, 5284491,
    6658042, 8388607, 10568983, 13316085, 16777216};
constexpr int LASTIDX = (int)(sizeof(RANGE) / sizeof(RANGE[0]));

typedef unsigned __int128 u128;

// bits needed by values below `size` in the format's count: the smallest b with 2^b > size
int bits_of(unsigned size) {
    int b = 0;
    unsigned long long v = 1;
    while (size >= v && b < 32) {
        b++;
        v <<= 1;
    }
    return b;
}

// the format's bit count for a triple with ranges s[0..2]: 8 per byte of the product below the
// top byte, plus the bits of the top byte (of the product itself, not product - 1)
int bits_of3(const unsigned s[3]) {
    u128 p = (u128)s[0] * s[1] * s[2];
    int bytes = 0;
    while ((p >> 8) != 0) {
        p >>= 8;
        bytes++;
    }
    int b = 0;
    unsigned top = (unsigned)p, v = 1;
    while (top >= v) {
        b++;
        v <<= 1;
    }
    return b + 8 * bytes;
}

struct BitReader {
    const unsigned char *p;
    size_t n, pos = 0;   // pos in bits
    bool bad = false;
    unsigned get(int nb) {   // nb <= 32, most significant bit first
        unsigned long long v = 0;
        for (int i = 0; i < nb; i++) {
            const size_t byte = pos >> 3;
            if (byte >= n) { bad = true; return 0; }
            v = (v << 1) | ((p[byte] >> (7 - (pos & 7))) & 1u);
            pos++;
        }
        return (unsigned)v;
    }
    // a mixed-radix triple over nb bits: 8-bit groups from the least significant byte up,
    // the last group holding the remaining high bits
    void triple(int nb, const unsigned s[3], int out[3]) {
        u128 v = 0;
        int shift = 0;
        while (nb > 8) {
            v |= (u128)get(8) << shift;
            shift += 8;
            nb -= 8;
        }
        if (nb > 0) v |= (u128)get(nb) << shift;
        out[2] = (int)(v % s[2]);
        v /= s[2];
        out[1] = (int)(v % s[1]);
        v /= s[1];
        out[0] = (int)v;
    }
};

struct BitWriter {
    std::vector<unsigned char> b;
    int used = 8;   // bits used in the last byte
    void put(unsigned v, int nb) {
        for (int i = nb - 1; i >= 0; i--) {
            if (used == 8) { b.push_back(0); used = 0; }
            b.back() |= (unsigned char)(((v >> i) & 1u) << (7 - used));
            used++;
        }
    }
    void triple(int nb, const unsigned s[3], const int c[3]) {
        u128 v = ((u128)(unsigned)c[0] * s[1] + (unsigned)c[1]) * s[2] + (unsigned)c[2];
        while (nb > 8) {
            put((unsigned)(v & 0xff), 8);
            v >>= 8;
            nb -= 8;
        }
        if (nb > 0) put((unsigned)v, nb);
    }
};

// ---- XDR primitives on a FILE ----
bool rd_u32(FILE *f, uint32_t *v) {
    unsigned char b[4];
    if (fread(b, 1, 4, f) != 4) return false;
    *v = ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3];
    return true;
}
bool rd_int(FILE *f, int *v) {
    uint32_t u;
    if (!rd_u32(f, &u)) return false;
    *v = (int)u;
    return true;
}
bool rd_float(FILE *f, float *v) {
    uint32_t u;
    if (!rd_u32(f, &u)) return false;
    memcpy(v, &u, 4);
    return true;
}
void wr_u32(std::vector<unsigned char> &o, uint32_t v) {
    o.push_back((unsigned char)(v >> 24));
    o.push_back((unsigned char)(v >> 16));
    o.push_back((unsigned char)(v >> 8));
    o.push_back((unsigned char)v);
}
void wr_int(std::vector<unsigned char> &o, int v) { wr_u32(o, (uint32_t)v); }
void wr_float(std::vector<unsigned char> &o, float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    wr_u32(o, u);
}

struct FrameHead {
    int natoms, step;
    float time, box[9];
};

bool read_head(FILE *f, FrameHead *h) {
    int magic;
    if (!rd_int(f, &magic)) return false;
    if (magic != XTC_MAGIC) return false;
    if (!rd_int(f, &h->natoms) || !rd_int(f, &h->step) || !rd_float(f, &h->time)) return false;
    for (int i = 0; i < 9; i++)
        if (!rd_float(f, &h->box[i])) return false;
    return true;
}

// Coordinates of one frame after its header: natoms again, then plain floats (up to 9 atoms)
// or the compressed form.  x: [natoms][3].  Returns false on a malformed frame.
bool read_coords(FILE *f, int natoms, float *x, float *prec_out) {
    int lsize;
    if (!rd_int(f, &lsize) || lsize != natoms) return false;
    if (natoms <= 9) {
        for (int i = 0; i < 3 * natoms; i++)
            if (!rd_float(f, &x[i])) return false;
        *prec_out = -1.f;
        return true;
    }
    float prec;
    int minint[3], maxint[3], smallidx, nbytes;
    if (!rd_float(f, &prec)) return false;
    for (int d = 0; d < 3; d++)
        if (!rd_int(f, &minint[d])) return false;
    for (int d = 0; d < 3; d++)
        if (!rd_int(f, &maxint[d])) return false;
    if (!rd_int(f, &smallidx) || !rd_int(f, &nbytes)) return false;
    if (!(prec > 0.f) || smallidx < FIRSTIDX || smallidx >= LASTIDX || nbytes < 0 || nbytes > natoms * 3 * 8 + 64) return false;
    for (int d = 0; d < 3; d++)
        if (maxint[d] < minint[d]) return false;
    std::vector<unsigned char> buf((size_t)((nbytes + 3) & ~3));
    if (!buf.empty() && fread(buf.data(), 1, buf.size(), f) != buf.size()) return false;
    unsigned sizeint[3], bitsizeint[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++) sizeint[d] = (unsigned)((long long)maxint[d] - minint[d] + 1);
    int bitsize = 0;
    if ((sizeint[0] | sizeint[1] | sizeint[2]) > 0xffffffu) {
        for (int d = 0; d < 3; d++) bitsizeint[d] = (unsigned)bits_of(sizeint[d]);
    } else {
        bitsize = bits_of3(sizeint);
    }
    int smaller = (int)RANGE[std::max(FIRSTIDX, smallidx - 1)] / 2;
    int smallnum = (int)RANGE[smallidx] / 2;
    unsigned sizesmall[3] = {RANGE[smallidx], RANGE[smallidx], RANGE[smallidx]};
    BitReader br{buf.data(), (size_t)nbytes};
    const float inv = 1.f / prec;
    int emitted = 0;
    auto emit = [&](const int c[3]) {
        if (emitted >= natoms) return;
        for (int d = 0; d < 3; d++) x[3 * emitted + d] = (float)c[d] * inv;
        emitted++;
    };
    int i = 0, run = 0;
    int cur[3], prev[3];
    while (i < natoms) {
        if (bitsize == 0) {
            for (int d = 0; d < 3; d++) cur[d] = (int)br.get((int)bitsizeint[d]);
        } else {
            br.triple(bitsize, sizeint, cur);
        }
        i++;
        for (int d = 0; d < 3; d++) {
            cur[d] += minint[d];
            prev[d] = cur[d];
        }
        int is_smaller = 0;
        if (br.get(1)) {
            run = (int)br.get(5);
            is_smaller = run % 3;
            run -= is_smaller;
            is_smaller--;
        }
        if (run > 0) {
            for (int k = 0; k < run; k += 3) {
                if (i >= natoms) return false;
                int t[3];
                br.triple(smallidx, sizesmall, t);
                i++;
                for (int d = 0; d < 3; d++) t[d] += prev[d] - smallnum;
                if (k == 0) {   // the first small atom precedes the large one
                    for (int d = 0; d < 3; d++) std::swap(t[d], prev[d]);
                    emit(prev);
                } else {
                    for (int d = 0; d < 3; d++) prev[d] = t[d];
                }
                emit(t);
            }
        } else {
            emit(cur);
        }
        smallidx += is_smaller;
        if (smallidx < FIRSTIDX || smallidx >= LASTIDX) return false;
        if (is_smaller < 0) {
            smallnum = smaller;
            smaller = smallidx > FIRSTIDX ? (int)RANGE[smallidx - 1] / 2 : 0;
        } else if (is_smaller > 0) {
            smaller = smallnum;
            smallnum = (int)RANGE[smallidx] / 2;
        }
        for (int d = 0; d < 3; d++) sizesmall[d] = RANGE[smallidx];
        if (br.bad) return false;
    }
    *prec_out = prec;
    return emitted == natoms;
}

int to_int(float v, float prec) {
    const float lf = v * prec;
    return (int)(lf >= 0.f ? lf + 0.5f : lf - 0.5f);
}

// Encoder: the inverse of read_coords.  Runs take consecutive atoms whose differences fit the
// small range (the first pair swapped as the format wants); the small index stays fixed,
// chosen so that at least half of the consecutive pairs fit.
void write_coords(std::vector<unsigned char> &o, int natoms, const float *x, float prec) {
    wr_int(o, natoms);
    if (natoms <= 9) {
        for (int i = 0; i < 3 * natoms; i++) wr_float(o, x[i]);
        return;
    }
    std::vector<int> c((size_t)natoms * 3);
    int minint[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, maxint[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int i = 0; i < natoms; i++)
        for (int d = 0; d < 3; d++) {
            const int v = to_int(x[3 * i + d], prec);
            c[3 * i + d] = v;
            minint[d] = std::min(minint[d], v);
            maxint[d] = std::max(maxint[d], v);
        }
    unsigned sizeint[3], bitsizeint[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++) sizeint[d] = (unsigned)((long long)maxint[d] - minint[d] + 1);
    int bitsize = 0;
    if ((sizeint[0] | sizeint[1] | sizeint[2]) > 0xffffffu) {
        for (int d = 0; d < 3; d++) bitsizeint[d] = (unsigned)bits_of(sizeint[d]);
    } else {
        bitsize = bits_of3(sizeint);
    }
    auto fits = [&](int idx, int a, int b) {   // atom a relative to atom b
        const long long half = RANGE[idx] / 2;
        for (int d = 0; d < 3; d++) {
            const long long v = (long long)c[3 * a + d] - c[3 * b + d] + half;
            if (v < 0 || v >= (long long)RANGE[idx]) return false;
        }
        return true;
    };
    int smallidx = LASTIDX - 1;
    for (int idx = FIRSTIDX; idx < LASTIDX; idx++) {
        int ok = 0;
        for (int i = 1; i < natoms; i++) ok += fits(idx, i, i - 1);
        if (2 * ok >= natoms - 1) { smallidx = idx; break; }
    }
    const int smallnum = (int)RANGE[smallidx] / 2;
    const unsigned sizesmall[3] = {RANGE[smallidx], RANGE[smallidx], RANGE[smallidx]};
    BitWriter bw;
    int run_state = 0;
    for (int i = 0; i < natoms;) {
        int m = 0;
        if (i + 1 < natoms && fits(smallidx, i, i + 1)) {
            m = 1;
            int ref = i;
            for (int j = i + 2; j < natoms && m < 10 && fits(smallidx, j, ref); j++) {
                m++;
                ref = j;
            }
        }
        const int big = m > 0 ? i + 1 : i;
        int rel[3];
        for (int d = 0; d < 3; d++) rel[d] = c[3 * big + d] - minint[d];
        if (bitsize == 0) {
            for (int d = 0; d < 3; d++) bw.put((unsigned)rel[d], (int)bitsizeint[d]);
        } else {
            bw.triple(bitsize, sizeint, rel);
        }
        if (3 * m == run_state) {
            bw.put(0, 1);
        } else {
            bw.put(1, 1);
            bw.put((unsigned)(3 * m + 1), 5);   // run x 3, small index unchanged
            run_state = 3 * m;
        }
        for (int q = 0; q < m; q++) {
            const int a = q == 0 ? i : i + 1 + q;
            const int b = q == 0 ? i + 1 : (q == 1 ? i : i + q);
            int t[3];
            for (int d = 0; d < 3; d++) t[d] = c[3 * a + d] - c[3 * b + d] + smallnum;
            bw.triple(smallidx, sizesmall, t);
        }
        i = m > 0 ? i + m + 1 : i + 1;
    }
    wr_float(o, prec);
    for (int d = 0; d < 3; d++) wr_int(o, minint[d]);
    for (int d = 0; d < 3; d++) wr_int(o, maxint[d]);
    wr_int(o, smallidx);
    wr_int(o, (int)bw.b.size());
    o.insert(o.end(), bw.b.begin(), bw.b.end());
    while (o.size() & 3) o.push_back(0);
}

// Byte offset of every frame (the random-access index of calcIR.cu:349), cached per path.
struct XtcIndex {
    std::vector<long> off;
    int natoms = 0;
    float t0 = 0, t1 = 0, prec1 = -1;
    long size = 0;
};

bool index_xtc(const char *path, XtcIndex *ix) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    ix->size = ftell(f);
    fseek(f, 0, SEEK_SET);
    ix->off.clear();
    bool ok = true;
    while (true) {
        const long pos = ftell(f);
        if (pos >= ix->size) break;
        FrameHead h;
        int lsize;
        if (!read_head(f, &h) || !rd_int(f, &lsize) || lsize != h.natoms) { ok = false; break; }
        if (ix->off.empty()) ix->natoms = h.natoms;
        else if (h.natoms != ix->natoms) { ok = false; break; }
        long skip;
        if (h.natoms <= 9) {
            skip = 12L * h.natoms;
            if (ix->off.size() == 1) ix->prec1 = -1.f;
        } else {
            float prec;
            int tmp[7], nbytes;
            if (!rd_float(f, &prec)) { ok = false; break; }
            for (int q = 0; q < 7; q++)
                if (!rd_int(f, &tmp[q])) { ok = false; break; }
            if (!ok || !rd_int(f, &nbytes) || nbytes < 0) { ok = false; break; }
            skip = (nbytes + 3) & ~3;
            if (ix->off.size() == 1) ix->prec1 = prec;
        }
        if (ix->off.empty()) ix->t0 = h.time;
        if (ix->off.size() == 1) ix->t1 = h.time;
        ix->off.push_back(pos);
        if (fseek(f, skip, SEEK_CUR) != 0 || ftell(f) > ix->size) { ok = false; break; }   // a cut frame
    }
    fclose(f);
    return ok && !ix->off.empty();
}

std::map<std::string, XtcIndex> g_index;

const XtcIndex *xtc_index(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return nullptr;
    fseek(f, 0, SEEK_END);
    const long size = ftell(f);
    fclose(f);
    auto it = g_index.find(path);
    if (it != g_index.end() && it->second.size == size) return &it->second;
    XtcIndex ix;
    if (!index_xtc(path, &ix)) return nullptr;
    g_index[path] = ix;
    return &g_index[path];
}

}  // namespace

bool cir_is_xtc(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    uint32_t m = 0;
    const bool ok = rd_u32(f, &m);
    fclose(f);
    return ok && m == (uint32_t)XTC_MAGIC;
}

// natoms, frame count and the frame spacing of calcIR.cu:341-346: the time difference of the
// first two frames rounded to the file's precision
int cir_xtc_info(const char *path, int *natoms, int *nframes, float *frame_dt) {
    const XtcIndex *ix = xtc_index(path);
    if (!ix) return cir_fail(CIR_ERR_IO, "%s: not a readable .xtc trajectory", path);
    if (natoms) *natoms = ix->natoms;
    if (nframes) *nframes = (int)ix->off.size();
    if (frame_dt) {
        float dt = 0.f;
        if (ix->off.size() > 1) {
            const float p = ix->prec1 > 0.f ? ix->prec1 : 1000.f;
            dt = (float)(round((ix->t1 - ix->t0) * p) / (1. * p));
        }
        *frame_dt = dt;
    }
    return CIR_OK;
}

int cir_xtc_read(const char *path, int first, int count, float *xyz, float *boxes, float *times) {
    const XtcIndex *ix = xtc_index(path);
    if (!ix) return cir_fail(CIR_ERR_IO, "%s: not a readable .xtc trajectory", path);
    if (first < 0 || count < 1 || first + count > (int)ix->off.size())
        return cir_fail(CIR_ERR_ARG, "%s: frames [%d, %d) outside the %zu frames", path, first, first + count, ix->off.size());
    FILE *f = fopen(path, "rb");
    if (!f) return cir_fail(CIR_ERR_IO, "%s: cannot open", path);
    for (int q = 0; q < count; q++) {
        FrameHead h;
        float prec;
        if (fseek(f, ix->off[first + q], SEEK_SET) != 0 || !read_head(f, &h) || h.natoms != ix->natoms ||
            !read_coords(f, h.natoms, xyz + (size_t)q * h.natoms * 3, &prec)) {
            fclose(f);
            return cir_fail(CIR_ERR_IO, "%s: frame %d is malformed", path, first + q);
        }
        if (boxes) {
            boxes[3 * q] = h.box[0];
            boxes[3 * q + 1] = h.box[4];
            boxes[3 * q + 2] = h.box[8];
        }
        if (times) times[q] = h.time;
    }
    fclose(f);
    return CIR_OK;
}

extern "C" int cir_xtc_write(const char *path, int natoms, int nframes, const float *xyz, const float *boxes,
                             const float *times, float precision) {
    if (!path || natoms < 1 || nframes < 1 || !xyz || !boxes || !(precision > 0.f))
        return cir_fail(CIR_ERR_ARG, "cir_xtc_write: bad argument");
    std::vector<unsigned char> o;
    for (int q = 0; q < nframes; q++) {
        wr_int(o, XTC_MAGIC);
        wr_int(o, natoms);
        wr_int(o, q);
        wr_float(o, times ? times[q] : 0.f);
        const float *b = boxes + 3 * q;
        const float box[9] = {b[0], 0, 0, 0, b[1], 0, 0, 0, b[2]};
        for (float v : box) wr_float(o, v);
        write_coords(o, natoms, xyz + (size_t)q * natoms * 3, precision);
    }
    FILE *f = fopen(path, "wb");
    if (!f) return cir_fail(CIR_ERR_IO, "%s: cannot create", path);
    const bool ok = fwrite(o.data(), 1, o.size(), f) == o.size();
    fclose(f);
    g_index.erase(path);
    return ok ? CIR_OK : cir_fail(CIR_ERR_IO, "%s: write failed", path);
}
