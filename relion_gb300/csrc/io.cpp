// io.cpp -- the data formats either side of the E-step: MRC image stacks
// (src/rwMRC.h) and STAR metadata tables (src/metadata_table.cpp).
//
// MRC: 1024-byte header (nx, ny, nz, mode at words 0-3, cell size a at word
// 10, mx at word 7, nsymbt at word 23), data after 1024 + nsymbt bytes;
// modes 0 (signed 8-bit, as the reference reads it since 3.1), 1 (int16),
// 2 (float32), 6 (uint16), 12 (float16) and 101 (4-bit, two pixels per
// byte, low nibble first); files written on a machine of the other byte
// order are recognised by an implausible mode / nx (the reference's
// SWAPTRIG test) and swapped.  Images are read straight into the caller's
// buffer (page-locked memory for the device upload), several threads in
// parallel for long reads, and converted to float32.
//
// STAR: data_ blocks holding either a loop_ table (_label #column lines,
// then rows) or label / value pairs; '#' comments; single- or double-quoted
// values.  Columns are kept as strings and converted on request.
#include "../../include/gbrelion.h"
#include "gbr_internal.h"

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kMrcHeader = 1024;
constexpr int kSwapTrig = 65535;  // a plausible mode / nx is far below this

uint32_t bswap32(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

int io_fail(int st, const std::string &m) {
    gbr::set_error_text(m);
    return st;
}

struct MrcInfo {
    int64_t nx = 0, ny = 0, nz = 0, mode = 0, nsymbt = 0;
    bool swapped = false;
    double pixel = 0.;
};

int read_mrc_info(const char *path, MrcInfo &info) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(GBR_ERR_INVALID, std::string("cannot open ") + path);
    unsigned char h[kMrcHeader];
    const size_t got = std::fread(h, 1, kMrcHeader, f);
    std::fclose(f);
    if (got != (size_t)kMrcHeader) return io_fail(GBR_ERR_INVALID, std::string("short MRC header in ") + path);
    auto word = [&](int i, bool swap) {
        uint32_t v;
        std::memcpy(&v, h + 4 * i, 4);
        return swap ? bswap32(v) : v;
    };
    int32_t mode = (int32_t)word(3, false), nx = (int32_t)word(0, false);
    bool swap = false;
    if (std::abs(mode) > kSwapTrig || std::abs(nx) > kSwapTrig) swap = true;
    info.swapped = swap;
    info.nx = (int32_t)word(0, swap);
    info.ny = (int32_t)word(1, swap);
    info.nz = (int32_t)word(2, swap);
    info.mode = (int32_t)word(3, swap);
    info.nsymbt = (int32_t)word(23, swap);
    const int32_t mx = (int32_t)word(7, swap);
    uint32_t ab = word(10, swap);
    float a;
    std::memcpy(&a, &ab, 4);
    info.pixel = mx > 0 ? (double)a / mx : 0.;
    if (info.nx <= 0 || info.ny <= 0 || info.nz <= 0 || info.nsymbt < 0)
        return io_fail(GBR_ERR_INVALID, std::string("bad MRC dimensions in ") + path);
    const int m = (int)info.mode;
    if (m != 0 && m != 1 && m != 2 && m != 6 && m != 12 && m != 101)
        return io_fail(GBR_ERR_UNSUPPORTED, "unsupported MRC mode " + std::to_string(m));
    return GBR_OK;
}

// bytes per image of a mode (mode 101 packs two pixels per byte)
int64_t image_bytes(const MrcInfo &i) {
    const int64_t px = i.nx * i.ny;
    switch (i.mode) {
    case 0: return px;
    case 1: case 6: case 12: return 2 * px;
    case 2: return 4 * px;
    case 101: return (px + 1) / 2;
    }
    return 0;
}

float half_to_float(uint16_t h) {
    const uint32_t s = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t bits;
    if (e == 0) {
        if (m == 0) {
            bits = s;
        } else {  // subnormal: normalise
            int ee = -1;
            uint32_t mm = m;
            do {
                ++ee;
                mm <<= 1;
            } while ((mm & 0x400u) == 0);
            bits = s | ((uint32_t)(127 - 15 - ee) << 23) | ((mm & 0x3ffu) << 13);
        }
    } else if (e == 31) {
        bits = s | 0x7f800000u | (m << 13);
    } else {
        bits = s | ((e + 127 - 15) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

void convert(const MrcInfo &info, const unsigned char *raw, int64_t npx, float *out) {
    switch (info.mode) {
    case 0:
        for (int64_t i = 0; i < npx; ++i) out[i] = (float)(int8_t)raw[i];
        break;
    case 1:
        for (int64_t i = 0; i < npx; ++i) {
            uint16_t v;
            std::memcpy(&v, raw + 2 * i, 2);
            if (info.swapped) v = (uint16_t)((v >> 8) | (v << 8));
            out[i] = (float)(int16_t)v;
        }
        break;
    case 6:
        for (int64_t i = 0; i < npx; ++i) {
            uint16_t v;
            std::memcpy(&v, raw + 2 * i, 2);
            if (info.swapped) v = (uint16_t)((v >> 8) | (v << 8));
            out[i] = (float)v;
        }
        break;
    case 12:
        for (int64_t i = 0; i < npx; ++i) {
            uint16_t v;
            std::memcpy(&v, raw + 2 * i, 2);
            if (info.swapped) v = (uint16_t)((v >> 8) | (v << 8));
            out[i] = half_to_float(v);
        }
        break;
    case 2:
        for (int64_t i = 0; i < npx; ++i) {
            uint32_t v;
            std::memcpy(&v, raw + 4 * i, 4);
            if (info.swapped) v = bswap32(v);
            std::memcpy(out + i, &v, 4);
        }
        break;
    case 101:
        for (int64_t i = 0; i < npx; ++i) {
            const unsigned char b = raw[i / 2];
            out[i] = (float)((i & 1) ? (b >> 4) : (b & 0x0f));
        }
        break;
    }
}

// ------------------------------------------------------------------ STAR
struct StarBlock {
    std::string name;
    bool loop = false;
    std::vector<std::string> labels;                  // without the leading '_'
    std::vector<std::vector<std::string>> rows;       // [row][col]
};

bool is_blank(const std::string &s) {
    return s.find_first_not_of(" \t\r\n") == std::string::npos;
}

// split a data line into tokens, honouring quotes
std::vector<std::string> tokens(const std::string &line) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
        if (i >= line.size() || line[i] == '#') break;
        if (line[i] == '"' || line[i] == '\'') {
            const char q = line[i++];
            const size_t j = line.find(q, i);
            out.push_back(line.substr(i, j == std::string::npos ? std::string::npos : j - i));
            i = j == std::string::npos ? line.size() : j + 1;
        } else {
            size_t j = i;
            while (j < line.size() && !std::isspace((unsigned char)line[j])) ++j;
            out.push_back(line.substr(i, j - i));
            i = j;
        }
    }
    return out;
}

}  // namespace

struct gbr_star {
    std::vector<StarBlock> blocks;
};

extern "C" {

int gbr_mrc_read_header(const char *path, gbr_mrc_header *out) {
    if (!path || !out) return io_fail(GBR_ERR_INVALID, "null argument");
    MrcInfo i;
    int s = read_mrc_info(path, i);
    if (s) return s;
    out->nx = i.nx;
    out->ny = i.ny;
    out->nz = i.nz;
    out->mode = i.mode;
    out->nsymbt = i.nsymbt;
    out->swapped = i.swapped ? 1 : 0;
    out->pixel_size = i.pixel;
    out->data_offset = kMrcHeader + i.nsymbt;
    return GBR_OK;
}

int gbr_mrc_read_images(const char *path, int64_t first, int64_t count, float *out, int nthreads) {
    if (!path || !out || first < 0 || count < 0) return io_fail(GBR_ERR_INVALID, "bad argument");
    MrcInfo info;
    int s = read_mrc_info(path, info);
    if (s) return s;
    if (first + count > info.nz) return io_fail(GBR_ERR_INVALID, "image range beyond the stack");
    const int64_t ib = image_bytes(info), npx = info.nx * info.ny;
    const int64_t base = kMrcHeader + info.nsymbt;
    nthreads = std::max(1, std::min<int>(nthreads > 0 ? nthreads : 1, (int)std::max<int64_t>(1, count)));
    std::vector<int> status(nthreads, GBR_OK);
    auto work = [&](int t) {
        const int64_t lo = count * t / nthreads, hi = count * (t + 1) / nthreads;
        if (lo >= hi) return;
        FILE *f = std::fopen(path, "rb");
        if (!f) {
            status[t] = GBR_ERR_INVALID;
            return;
        }
        std::vector<unsigned char> raw((size_t)ib);
        if (std::fseek(f, (long)(base + (first + lo) * ib), SEEK_SET) != 0) status[t] = GBR_ERR_INVALID;
        for (int64_t k = lo; k < hi && status[t] == GBR_OK; ++k) {
            if (info.mode == 2 && !info.swapped) {
                // float32: straight into the destination
                if (std::fread(out + k * npx, 1, (size_t)ib, f) != (size_t)ib) status[t] = GBR_ERR_INVALID;
            } else {
                if (std::fread(raw.data(), 1, (size_t)ib, f) != (size_t)ib) status[t] = GBR_ERR_INVALID;
                else convert(info, raw.data(), npx, out + k * npx);
            }
        }
        std::fclose(f);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    for (int v : status)
        if (v != GBR_OK) return io_fail(GBR_ERR_INVALID, std::string("short read in ") + path);
    return GBR_OK;
}

int gbr_mrc_write_stack(const char *path, const float *data, int64_t nx, int64_t ny, int64_t nz,
                        double pixel_size) {
    if (!path || !data || nx <= 0 || ny <= 0 || nz <= 0) return io_fail(GBR_ERR_INVALID, "bad argument");
    unsigned char h[kMrcHeader];
    std::memset(h, 0, sizeof h);
    auto put_i = [&](int w, int32_t v) { std::memcpy(h + 4 * w, &v, 4); };
    auto put_f = [&](int w, float v) { std::memcpy(h + 4 * w, &v, 4); };
    const int64_t npx = nx * ny * nz;
    float mn = data[0], mx = data[0];
    double sum = 0.;
    for (int64_t i = 0; i < npx; ++i) {
        mn = std::min(mn, data[i]);
        mx = std::max(mx, data[i]);
        sum += data[i];
    }
    put_i(0, (int32_t)nx);
    put_i(1, (int32_t)ny);
    put_i(2, (int32_t)nz);
    put_i(3, 2);
    put_i(7, (int32_t)nx);
    put_i(8, (int32_t)ny);
    put_i(9, (int32_t)nz);
    put_f(10, (float)(pixel_size * nx));
    put_f(11, (float)(pixel_size * ny));
    put_f(12, (float)(pixel_size * nz));
    put_f(13, 90.f);
    put_f(14, 90.f);
    put_f(15, 90.f);
    put_i(16, 1);
    put_i(17, 2);
    put_i(18, 3);
    put_f(19, mn);
    put_f(20, mx);
    put_f(21, (float)(sum / (double)npx));
    put_i(22, nz > 1 ? 0 : 1);
    std::memcpy(h + 4 * 52, "MAP ", 4);
    const unsigned char stamp[4] = {0x44, 0x44, 0x00, 0x00};  // little-endian machine stamp
    std::memcpy(h + 4 * 53, stamp, 4);
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(GBR_ERR_INVALID, std::string("cannot create ") + path);
    bool ok = std::fwrite(h, 1, kMrcHeader, f) == (size_t)kMrcHeader;
    ok = ok && std::fwrite(data, sizeof(float), (size_t)npx, f) == (size_t)npx;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GBR_OK : io_fail(GBR_ERR_INVALID, std::string("write failed: ") + path);
}

int gbr_star_read(const char *path, gbr_star **out) {
    if (!path || !out) return io_fail(GBR_ERR_INVALID, "null argument");
    std::ifstream in(path);
    if (!in) return io_fail(GBR_ERR_INVALID, std::string("cannot open ") + path);
    std::unique_ptr<gbr_star> st(new gbr_star());
    StarBlock *cur = nullptr;
    bool in_loop_header = false;
    std::string line;
    while (std::getline(in, line)) {
        std::vector<std::string> tk = tokens(line);
        if (tk.empty()) {
            continue;
        }
        const std::string &t0 = tk[0];
        if (t0.compare(0, 5, "data_") == 0) {
            st->blocks.emplace_back();
            cur = &st->blocks.back();
            cur->name = t0.substr(5);
            in_loop_header = false;
            continue;
        }
        if (!cur) continue;  // text before the first block
        if (t0 == "loop_") {
            cur->loop = true;
            in_loop_header = true;
            continue;
        }
        if (t0[0] == '_') {
            if (cur->loop && in_loop_header) {
                cur->labels.push_back(t0.substr(1));  // "_rlnX #n"
            } else {
                // label / value pair of a non-loop block
                cur->labels.push_back(t0.substr(1));
                if (cur->rows.empty()) cur->rows.emplace_back();
                cur->rows[0].push_back(tk.size() > 1 ? tk[1] : std::string());
            }
            continue;
        }
        if (cur->loop) {
            in_loop_header = false;
            if (tk.size() != cur->labels.size())
                return io_fail(GBR_ERR_INVALID, "STAR row with " + std::to_string(tk.size()) + " values for " +
                                                    std::to_string(cur->labels.size()) + " columns in block " +
                                                    cur->name);
            cur->rows.push_back(tk);
        }
    }
    *out = st.release();
    return GBR_OK;
}

int64_t gbr_star_num_blocks(const gbr_star *s) { return s ? (int64_t)s->blocks.size() : 0; }

int gbr_star_block_info(const gbr_star *s, int64_t ib, char *name, size_t len, int64_t *ncols, int64_t *nrows,
                        int *is_loop) {
    if (!s || ib < 0 || ib >= (int64_t)s->blocks.size()) return io_fail(GBR_ERR_INVALID, "bad block");
    const StarBlock &b = s->blocks[ib];
    if (name && len) {
        std::strncpy(name, b.name.c_str(), len - 1);
        name[len - 1] = 0;
    }
    if (ncols) *ncols = (int64_t)b.labels.size();
    if (nrows) *nrows = (int64_t)b.rows.size();
    if (is_loop) *is_loop = b.loop ? 1 : 0;
    return GBR_OK;
}

int gbr_star_column_name(const gbr_star *s, int64_t ib, int64_t ic, char *name, size_t len) {
    if (!s || ib < 0 || ib >= (int64_t)s->blocks.size() || !name || !len) return io_fail(GBR_ERR_INVALID, "bad block");
    const StarBlock &b = s->blocks[ib];
    if (ic < 0 || ic >= (int64_t)b.labels.size()) return io_fail(GBR_ERR_INVALID, "bad column");
    std::strncpy(name, b.labels[ic].c_str(), len - 1);
    name[len - 1] = 0;
    return GBR_OK;
}

static int find_col(const gbr_star *s, int64_t ib, const char *label) {
    if (!s || ib < 0 || ib >= (int64_t)s->blocks.size() || !label) return -1;
    const StarBlock &b = s->blocks[ib];
    const char *l = label[0] == '_' ? label + 1 : label;
    for (size_t c = 0; c < b.labels.size(); ++c)
        if (b.labels[c] == l) return (int)c;
    return -1;
}

int gbr_star_column_double(const gbr_star *s, int64_t ib, const char *label, double *out) {
    const int c = find_col(s, ib, label);
    if (c < 0 || !out) return io_fail(GBR_ERR_INVALID, std::string("no column ") + (label ? label : "?"));
    const StarBlock &b = s->blocks[ib];
    for (size_t r = 0; r < b.rows.size(); ++r) {
        char *end = nullptr;
        const std::string &v = b.rows[r][c];
        out[r] = std::strtod(v.c_str(), &end);
        if (end == v.c_str()) return io_fail(GBR_ERR_INVALID, "non-numeric value '" + v + "' in column " + label);
    }
    return GBR_OK;
}

int gbr_star_value_string(const gbr_star *s, int64_t ib, const char *label, int64_t row, char *buf, size_t len) {
    const int c = find_col(s, ib, label);
    if (c < 0 || !buf || !len) return io_fail(GBR_ERR_INVALID, std::string("no column ") + (label ? label : "?"));
    const StarBlock &b = s->blocks[ib];
    if (row < 0 || row >= (int64_t)b.rows.size()) return io_fail(GBR_ERR_INVALID, "bad row");
    std::strncpy(buf, b.rows[row][c].c_str(), len - 1);
    buf[len - 1] = 0;
    return GBR_OK;
}

void gbr_star_free(gbr_star *s) { delete s; }

}  // extern "C"
