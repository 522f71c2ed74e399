// hb_io.cu — NPY files as hyburn reads and writes them (io.rs:19-125), and the batch sweep's
// per-subnetwork temporal-average files tavg_sub{i}.npy (cli.rs:947-970). Host code only.
//
// Writer (io.rs:88-125): magic "\x93NUMPY", version 1.0, a little-endian u16 header length, the header
//   {'descr': '<f4', 'fortran_order': False, 'shape': (d0, d1, ...) }
// (a one-dimensional shape is written "(d0,)") padded with spaces so that 10 + header + newline is a
// multiple of 64, a newline, then the values as little-endian f32.
// Reader (io.rs:25-83, 150-228): checks the magic, takes the header length from two bytes (major
// version < 2) or four, finds the 'shape' and 'descr' values with a scanner that skips keys inside
// string literals, accepts the descriptors '<f4', '|f4', 'f4' and '<f8' (f8 values are rounded to
// f32), ignores 'fortran_order', and returns every whole value after the header (so trailing bytes
// beyond the shape's product come back as extra values, as in the reference).
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "hyburn_gb300.h"

void hb_internal_set_error(const char* msg);  // hb_engine.cu: the text hb_last_error returns

namespace {

hb_status io_fail(hb_status st, const std::string& msg) {
    hb_internal_set_error(msg.c_str());
    return st;
}

std::string os_error_text(int err) { return std::string(strerror(err)) + " (os error " + std::to_string(err) + ")"; }

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && is_ws(s[a])) a++;
    while (b > a && is_ws(s[b - 1])) b--;
    return s.substr(a, b - a);
}

// The value of a quoted key 'key': in an NPY header: a parenthesised tuple (its contents, trimmed)
// or a quoted string (its contents). Quote characters outside a key match toggle an in-string
// flag, and keys are only matched outside strings. Returns 0 when found, 1 when absent, 2 when a
// tuple is not closed.
int quoted_value(const std::string& h, const std::string& key, std::string& out) {
    const size_t n = h.size(), kl = key.size();
    bool in_string = false;
    for (size_t i = 0; i < n; i++) {
        const char ch = h[i];
        if (!in_string && (ch == '\'' || ch == '"')) {
            const char q = ch;
            if (i + 1 + kl + 1 < n && h.compare(i + 1, kl, key) == 0 && h[i + 1 + kl] == q && h[i + 1 + kl + 1] == ':') {
                size_t v = i + 1 + kl + 2;
                while (v < n && is_ws(h[v])) v++;
                if (v < n && h[v] == '(') {
                    int depth = 0;
                    for (size_t k = v; k < n; k++) {
                        if (h[k] == '(') depth++;
                        if (h[k] == ')') depth--;
                        if (depth == 0 && h[k] == ')') {
                            out = trim(h.substr(v + 1, k - v - 1));
                            return 0;
                        }
                    }
                    return 2;
                } else if (v < n && (h[v] == '\'' || h[v] == '"')) {
                    const size_t end = h.find(h[v], v + 1);
                    if (end != std::string::npos) {
                        out = h.substr(v + 1, end - v - 1);
                        return 0;
                    }
                }
            }
        }
        if (ch == '\'' || ch == '"') in_string = !in_string;
    }
    return 1;
}

// one shape entry as an unsigned integer: an optional '+' and decimal digits
bool parse_dim(const std::string& s, uint64_t& v, std::string& why) {
    size_t i = (!s.empty() && s[0] == '+') ? 1 : 0;
    if (i == s.size()) { why = "invalid digit found in string"; return false; }
    v = 0;
    for (; i < s.size(); i++) {
        if (s[i] < '0' || s[i] > '9') { why = "invalid digit found in string"; return false; }
        const uint64_t d = (uint64_t)(s[i] - '0');
        if (v > (UINT64_MAX - d) / 10) { why = "number too large to fit in target type"; return false; }
        v = v * 10 + d;
    }
    return true;
}

hb_status parse_shape(const std::string& header, std::vector<uint64_t>& shape) {
    std::string inner;
    const int r = quoted_value(header, "shape", inner);
    if (r == 1) return io_fail(HB_ERR_INVALID_STATE, "No 'shape' key in NPY header");
    if (r == 2) return io_fail(HB_ERR_INVALID_STATE, "Failed to parse NPY shape: unclosed tuple");
    shape.clear();
    size_t p = 0;
    while (p <= inner.size()) {
        size_t c = inner.find(',', p);
        if (c == std::string::npos) c = inner.size();
        const std::string part = trim(inner.substr(p, c - p));
        if (!part.empty()) {
            uint64_t v;
            std::string why;
            if (!parse_dim(part, v, why)) return io_fail(HB_ERR_INVALID_STATE, "Failed to parse NPY shape: " + why);
            shape.push_back(v);
        }
        p = c + 1;
    }
    return HB_OK;
}

uint32_t le32(const unsigned char* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }

bool read_file(const char* path, std::vector<unsigned char>& buf, int& err) {
    FILE* f = fopen(path, "rb");
    if (!f) { err = errno; return false; }
    unsigned char tmp[1 << 16];
    size_t got;
    while ((got = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
    err = ferror(f) ? EIO : 0;
    fclose(f);
    return err == 0;
}

hb_status write_npy(const char* path, const float* data, const int64_t* shape, int32_t ndim) {
    uint64_t total = 1;
    for (int i = 0; i < ndim; i++) {
        if (shape[i] < 0) return io_fail(HB_ERR_INVALID_STATE, "negative NPY dimension");
        total *= (uint64_t)shape[i];
    }
    std::string sh;
    if (ndim == 1) sh = "(" + std::to_string(shape[0]) + ",)";
    else {
        sh = "(";
        for (int i = 0; i < ndim; i++) sh += (i ? ", " : "") + std::to_string(shape[i]);
        sh += ")";
    }
    std::string header = "{'descr': '<f4', 'fortran_order': False, 'shape': " + sh + " }";
    const size_t rem = (header.size() + 10 + 1) % 64;
    header.append(rem ? 64 - rem : 0, ' ');
    header.push_back('\n');
    if (header.size() > 0xffff) return io_fail(HB_ERR_INVALID_STATE, "NPY header longer than 65535 bytes");
    FILE* f = fopen(path, "wb");
    if (!f) return io_fail(HB_ERR_IO, os_error_text(errno));
    std::vector<unsigned char> out;
    out.reserve(10 + header.size() + total * 4);
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    out.insert(out.end(), magic, magic + 8);
    out.push_back((unsigned char)(header.size() & 0xff));
    out.push_back((unsigned char)(header.size() >> 8));
    out.insert(out.end(), header.begin(), header.end());
    for (uint64_t i = 0; i < total; i++) {
        uint32_t u;
        memcpy(&u, data + i, 4);
        const unsigned char b[4] = {(unsigned char)u, (unsigned char)(u >> 8), (unsigned char)(u >> 16), (unsigned char)(u >> 24)};
        out.insert(out.end(), b, b + 4);
    }
    const size_t put = fwrite(out.data(), 1, out.size(), f);
    const int werr = (put != out.size()) ? (errno ? errno : EIO) : 0;
    if (fclose(f) != 0 && !werr) return io_fail(HB_ERR_IO, os_error_text(errno));
    if (werr) return io_fail(HB_ERR_IO, os_error_text(werr));
    return HB_OK;
}

}  // namespace

extern "C" {

hb_status hb_npy_write_f32(const char* path, const float* data, const int64_t* shape, int32_t ndim) {
    if (!path || ndim < 0 || (ndim > 0 && !shape)) return io_fail(HB_ERR_INVALID_STATE, "hb_npy_write_f32: bad arguments");
    uint64_t total = 1;
    for (int i = 0; i < ndim; i++) total *= (uint64_t)(shape[i] < 0 ? 0 : shape[i]);
    if (total > 0 && !data) return io_fail(HB_ERR_INVALID_STATE, "hb_npy_write_f32: no data");
    return write_npy(path, data, shape, ndim);
}

hb_status hb_npy_read_f32(const char* path, float* out, int64_t capacity, int64_t* shape, int32_t max_ndim,
                          int32_t* ndim, int64_t* n_values) {
    if (!path) return io_fail(HB_ERR_INVALID_STATE, "hb_npy_read_f32: no path");
    std::vector<unsigned char> buf;
    int err = 0;
    if (!read_file(path, buf, err)) return io_fail(HB_ERR_IO, os_error_text(err));
    static const unsigned char magic[6] = {0x93, 'N', 'U', 'M', 'P', 'Y'};
    // the reference indexes the fixed prefix without a length check (a panic on shorter files)
    if (buf.size() < 10 || memcmp(buf.data(), magic, 6) != 0) return io_fail(HB_ERR_INVALID_STATE, "Not a valid .npy file");
    const unsigned major = buf[6];
    size_t header_len;
    if (major < 2) header_len = 10 + ((size_t)buf[8] | ((size_t)buf[9] << 8));
    else {
        if (buf.size() < 12) return io_fail(HB_ERR_INVALID_STATE, "Not a valid .npy file");
        header_len = 12 + (size_t)le32(buf.data() + 8);
    }
    // the header text starts after the two-byte length field in both versions (io.rs:49)
    const size_t hend = header_len < buf.size() ? header_len : buf.size();
    const std::string header(reinterpret_cast<const char*>(buf.data()) + 10, hend > 10 ? hend - 10 : 0);
    std::vector<uint64_t> dims;
    hb_status s = parse_shape(header, dims);
    if (s) return s;
    std::string descr;
    if (quoted_value(header, "descr", descr) != 0) return io_fail(HB_ERR_INVALID_STATE, "No 'descr' key in NPY header");
    if (descr != "<f4" && descr != "|f4" && descr != "f4" && descr != "<f8")
        return io_fail(HB_ERR_INVALID_STATE, "Unsupported NPY dtype descriptor: '" + descr + "', only f32/f64 supported");
    uint64_t total = 1;
    for (uint64_t d : dims) total = (d != 0 && total > UINT64_MAX / d) ? UINT64_MAX : total * d;
    const bool f8 = descr == "<f8";
    const size_t esz = f8 ? 8 : 4;
    const size_t avail = header_len < buf.size() ? buf.size() - header_len : 0;
    if ((uint64_t)avail / esz < total)
        return io_fail(HB_ERR_INVALID_STATE, f8 ? "NPY data truncated (f64)" : "NPY data truncated (f32)");
    const int64_t n = (int64_t)(avail / esz);
    if (ndim) *ndim = (int32_t)dims.size();
    if (n_values) *n_values = n;
    if (shape) {
        if ((int32_t)dims.size() > max_ndim) return io_fail(HB_ERR_INVALID_STATE, "NPY array has more dimensions than the shape buffer");
        for (size_t i = 0; i < dims.size(); i++) shape[i] = (int64_t)dims[i];
    }
    if (!out) return HB_OK;  // size query
    if (capacity < n) return io_fail(HB_ERR_INVALID_STATE, "output buffer holds fewer values than the NPY file");
    const unsigned char* p = buf.data() + header_len;
    for (int64_t i = 0; i < n; i++) {
        if (f8) {
            const uint64_t u = (uint64_t)le32(p + 8 * i) | ((uint64_t)le32(p + 8 * i + 4) << 32);
            double d;
            memcpy(&d, &u, 8);
            out[i] = (float)d;
        } else {
            const uint32_t u = le32(p + 4 * i);
            memcpy(out + i, &u, 4);
        }
    }
    return HB_OK;
}

}  // extern "C"

// create_dir_all: every missing directory of `dir`
hb_status hb_io_make_dirs(const std::string& dir) {
    std::string cur;
    size_t p = 0;
    while (p <= dir.size()) {
        size_t c = dir.find('/', p);
        if (c == std::string::npos) c = dir.size();
        cur = dir.substr(0, c);
        if (!cur.empty()) {
            struct stat st;
            if (stat(cur.c_str(), &st) != 0) {
                if (mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) return io_fail(HB_ERR_IO, os_error_text(errno));
            } else if (!S_ISDIR(st.st_mode)) {
                return io_fail(HB_ERR_IO, os_error_text(EEXIST));
            }
        }
        p = c + 1;
    }
    return HB_OK;
}

hb_status hb_io_write_npy(const std::string& path, const float* data, const std::vector<int64_t>& shape) {
    return write_npy(path.c_str(), data, shape.data(), (int32_t)shape.size());
}
