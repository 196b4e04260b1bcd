// .npy / .npz reader and .npy writer (see npy.h).  The .npz reader walks the zip central
// directory (zip64 records included, which numpy.savez writes for every member) and
// accepts stored (uncompressed) members only.
#include "npy.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace bpgb {

namespace {

uint16_t rd16(const unsigned char *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
uint32_t rd32(const unsigned char *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
uint64_t rd64(const unsigned char *p) { return (uint64_t)rd32(p) | ((uint64_t)rd32(p + 4) << 32); }

bool read_file(const std::string &path, std::vector<unsigned char> *buf, std::string *why) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        if (why) *why = "cannot open " + path;
        return false;
    }
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0, std::ios::beg);
    buf->resize((size_t)n);
    if (n > 0 && !f.read((char *)buf->data(), n)) {
        if (why) *why = "cannot read " + path;
        return false;
    }
    return true;
}

// Value of key `k` in the npy header dict (the text up to the next top-level ',' or '}').
bool dict_value(const std::string &h, const std::string &k, std::string *v) {
    const size_t p = h.find("'" + k + "'");
    if (p == std::string::npos) return false;
    size_t c = h.find(':', p);
    if (c == std::string::npos) return false;
    c++;
    int depth = 0;
    size_t e = c;
    for (; e < h.size(); e++) {
        const char ch = h[e];
        if (ch == '(' || ch == '[') depth++;
        if (ch == ')' || ch == ']') depth--;
        if (depth == 0 && (ch == ',' || ch == '}')) break;
    }
    *v = h.substr(c, e - c);
    const size_t a = v->find_first_not_of(" \t");
    const size_t b = v->find_last_not_of(" \t");
    *v = a == std::string::npos ? "" : v->substr(a, b - a + 1);
    return true;
}

}  // namespace

uint64_t NpyArray::count() const {
    uint64_t n = 1;
    for (uint64_t s : shape) n *= s;
    return n;
}

uint32_t NpyArray::itemsize() const { return (uint32_t)std::atoi(descr.c_str() + 2); }

double NpyArray::at(uint64_t i) const {
    const unsigned char *p = bytes.data() + i * itemsize();
    const char kind = descr[1];
    const uint32_t sz = itemsize();
    if (kind == 'f' && sz == 4) {
        float v;
        std::memcpy(&v, p, 4);
        return v;
    }
    if (kind == 'f' && sz == 8) {
        double v;
        std::memcpy(&v, p, 8);
        return v;
    }
    if (kind == 'c' && sz == 8) {
        float v;
        std::memcpy(&v, p, 4);
        return v;
    }
    if (kind == 'i' && sz == 4) return (double)(int32_t)rd32(p);
    if (kind == 'i' && sz == 8) return (double)(int64_t)rd64(p);
    if (kind == 'u' && sz == 4) return (double)rd32(p);
    if (kind == 'u' && sz == 8) return (double)rd64(p);
    if ((kind == 'u' || kind == 'b') && sz == 1) return (double)p[0];
    return 0.0;
}

std::vector<float> NpyArray::as_float() const {
    std::vector<float> out(count());
    if (descr == "<f4") {
        std::memcpy(out.data(), bytes.data(), out.size() * 4);
        return out;
    }
    for (uint64_t i = 0; i < out.size(); i++) out[i] = (float)at(i);
    return out;
}

bool npy_parse(const unsigned char *data, size_t size, NpyArray *out, std::string *why) {
    auto fail = [&](const std::string &m) {
        if (why) *why = m;
        return false;
    };
    if (size < 10 || std::memcmp(data, "\x93NUMPY", 6) != 0) return fail("not an .npy image");
    const int major = data[6];
    size_t hlen, hoff;
    if (major == 1) {
        hlen = rd16(data + 8);
        hoff = 10;
    } else if (major == 2 || major == 3) {
        if (size < 12) return fail("truncated .npy header");
        hlen = rd32(data + 8);
        hoff = 12;
    } else {
        return fail("unknown .npy version");
    }
    if (hoff + hlen > size) return fail("truncated .npy header");
    const std::string h((const char *)data + hoff, hlen);
    std::string descr, order, shape;
    if (!dict_value(h, "descr", &descr) || !dict_value(h, "fortran_order", &order) ||
        !dict_value(h, "shape", &shape))
        return fail("malformed .npy header");
    if (descr.size() < 4 || (descr[0] != '\'' && descr[0] != '"'))
        return fail("unsupported dtype " + descr);
    descr = descr.substr(1, descr.size() - 2);
    if (descr == "|u1" || descr == "|b1" || descr == "|i1") descr = std::string("<") + descr[1] + "1";
    static const char *kOk[] = {"<f4", "<f8", "<i4", "<i8", "<u4", "<u8", "<u1", "<b1", "<c8"};
    bool ok = false;
    for (const char *k : kOk) ok = ok || descr == k;
    if (!ok) return fail("unsupported dtype " + descr + " (little-endian f4/f8/i4/i8/u4/u1/b1/c8)");
    if (order != "False") return fail("Fortran-ordered arrays are not supported");
    out->descr = descr;
    out->shape.clear();
    std::string s = shape;
    for (char &c : s)
        if (c == '(' || c == ')' || c == ',') c = ' ';
    std::istringstream in(s);
    uint64_t d;
    while (in >> d) out->shape.push_back(d);
    const uint64_t nbytes = out->count() * out->itemsize();
    const size_t doff = hoff + hlen;
    if (doff + nbytes > size) return fail("truncated .npy data");
    out->bytes.assign(data + doff, data + doff + nbytes);
    return true;
}

bool npy_load(const std::string &path, NpyArray *out, std::string *why) {
    std::vector<unsigned char> buf;
    if (!read_file(path, &buf, why)) return false;
    if (!npy_parse(buf.data(), buf.size(), out, why)) {
        if (why) *why = path + ": " + *why;
        return false;
    }
    return true;
}

bool npz_load(const std::string &path, std::map<std::string, NpyArray> *out, std::string *why) {
    std::vector<unsigned char> buf;
    if (!read_file(path, &buf, why)) return false;
    auto fail = [&](const std::string &m) {
        if (why) *why = path + ": " + m;
        return false;
    };
    const size_t n = buf.size();
    if (n < 22) return fail("not a zip archive");
    // end of central directory (comment up to 64 KB)
    size_t eocd = std::string::npos;
    for (size_t i = n - 22 + 1; i-- > 0 && n - i <= 22 + 65535;) {
        if (rd32(&buf[i]) == 0x06054b50u) {
            eocd = i;
            break;
        }
    }
    if (eocd == std::string::npos) return fail("zip end-of-directory record not found");
    uint64_t entries = rd16(&buf[eocd + 10]);
    uint64_t cd_off = rd32(&buf[eocd + 16]);
    if (cd_off == 0xFFFFFFFFu || entries == 0xFFFFu) {
        if (eocd < 20 || rd32(&buf[eocd - 20]) != 0x07064b50u) return fail("zip64 locator missing");
        const uint64_t z64 = rd64(&buf[eocd - 20 + 8]);
        if (z64 + 56 > n || rd32(&buf[z64]) != 0x06064b50u) return fail("zip64 record missing");
        entries = rd64(&buf[z64 + 32]);
        cd_off = rd64(&buf[z64 + 48]);
    }
    size_t p = (size_t)cd_off;
    out->clear();
    for (uint64_t e = 0; e < entries; e++) {
        if (p + 46 > n || rd32(&buf[p]) != 0x02014b50u) return fail("bad central directory");
        const uint16_t method = rd16(&buf[p + 10]);
        uint64_t csize = rd32(&buf[p + 20]);
        uint64_t usize = rd32(&buf[p + 24]);
        const uint16_t nlen = rd16(&buf[p + 28]), xlen = rd16(&buf[p + 30]), clen = rd16(&buf[p + 32]);
        uint64_t loff = rd32(&buf[p + 42]);
        if (p + 46 + nlen + xlen > n) return fail("bad central directory entry");
        std::string name((const char *)&buf[p + 46], nlen);
        // zip64 extra field: the 0xFFFFFFFF fields, in order usize, csize, offset
        size_t x = p + 46 + nlen, xe = x + xlen;
        while (x + 4 <= xe) {
            const uint16_t id = rd16(&buf[x]), sz = rd16(&buf[x + 2]);
            if (id == 0x0001) {
                size_t q = x + 4;
                if (usize == 0xFFFFFFFFu && q + 8 <= x + 4 + sz) usize = rd64(&buf[q]), q += 8;
                if (csize == 0xFFFFFFFFu && q + 8 <= x + 4 + sz) csize = rd64(&buf[q]), q += 8;
                if (loff == 0xFFFFFFFFu && q + 8 <= x + 4 + sz) loff = rd64(&buf[q]), q += 8;
            }
            x += 4 + sz;
        }
        p += 46 + nlen + xlen + clen;
        if (method != 0) return fail(name + " is compressed (use numpy.savez, not savez_compressed)");
        if (loff + 30 > n || rd32(&buf[loff]) != 0x04034b50u) return fail(name + ": bad local header");
        const size_t data = (size_t)loff + 30 + rd16(&buf[loff + 26]) + rd16(&buf[loff + 28]);
        if (csize != usize || data + csize > n) return fail(name + ": bad member size");
        NpyArray a;
        std::string w;
        if (!npy_parse(&buf[data], (size_t)csize, &a, &w)) {
            if (w.compare(0, 17, "unsupported dtype") == 0) continue;  // e.g. text members
            return fail(name + ": " + w);
        }
        if (name.size() > 4 && name.compare(name.size() - 4, 4, ".npy") == 0)
            name = name.substr(0, name.size() - 4);
        (*out)[name] = std::move(a);
    }
    return true;
}

bool npy_save_f32(const std::string &path, const float *data, const std::vector<uint64_t> &shape,
                  std::string *why) {
    std::string sh = "(";
    for (size_t i = 0; i < shape.size(); i++) sh += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
    sh += ")";
    std::string h = "{'descr': '<f4', 'fortran_order': False, 'shape': " + sh + ", }";
    const size_t total = 10 + h.size() + 1;
    h.append((64 - total % 64) % 64, ' ');
    h.push_back('\n');
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) {
        if (why) *why = "cannot write " + path;
        return false;
    }
    const unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0,
                                   (unsigned char)(h.size() & 0xff), (unsigned char)(h.size() >> 8)};
    f.write((const char *)pre, 10);
    f.write(h.data(), (std::streamsize)h.size());
    uint64_t count = 1;
    for (uint64_t s : shape) count *= s;
    f.write((const char *)data, (std::streamsize)(count * 4));
    if (!f) {
        if (why) *why = "write failed: " + path;
        return false;
    }
    return true;
}

}  // namespace bpgb
