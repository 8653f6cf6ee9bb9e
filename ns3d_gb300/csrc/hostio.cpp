// hostio.cpp -- ini parser, .vti codec (zlib), shared by the C-ABI and the CLI.
#include "hostio.h"

#include <zlib.h>

#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>

namespace ns3d {

// ============================ ini ==========================================
// Behaviour of ReadInput, src/navierstokes3D.cxx:266-463: one "key = value"
// per line, keys case-insensitive, '#' comments (a '#' starts an inline
// comment only at the start of the value or after whitespace), unknown keys
// warn, a malformed value or a missing 'input' is fatal.  The key compared as
// "deltaRMR" after lowercasing never matches (src/navierstokes3D.cxx:342), so
// deltaRMR always keeps its default; that is reproduced.  One key is added:
// precision = FP64 | MIXED | MIXED_MG selects the arithmetic (and, for
// MIXED_MG, the preconditioner) of the inner solves.
static std::string trim(const std::string &s) {
    const char *ws = " \t\r\n";
    size_t b = s.find_first_not_of(ws);
    if (b == std::string::npos) return std::string();
    size_t e = s.find_last_not_of(ws);
    return s.substr(b, e - b + 1);
}
static std::string lower(std::string s) {
    for (char &c : s)
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    return s;
}
static std::string upper(std::string s) {
    for (char &c : s)
        if (c >= 'a' && c <= 'z') c = (char)(c - 'a' + 'A');
    return s;
}
static bool parse_double(const std::string &s, double &out) {
    if (s.empty()) return false;
    size_t pos = 0;
    try {
        out = std::stod(s, &pos);
    } catch (...) {
        return false;
    }
    return pos == s.size();
}
static bool parse_int(const std::string &s, int &out) {
    if (s.empty()) return false;
    size_t pos = 0;
    try {
        out = std::stoi(s, &pos);
    } catch (...) {
        return false;
    }
    return pos == s.size();
}
static std::string strip_comment(const std::string &v) {
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i] == '#' && (i == 0 || std::isspace((unsigned char)v[i - 1]))) return trim(v.substr(0, i));
    return trim(v);
}

const char *method_name(int m) {
    switch (m) {
        case NS3D_SIMPLER: return "SIMPLER";
        case NS3D_SIMPLERR: return "SIMPLERR";
        case NS3D_IDEAL: return "IDEAL";
        default: return "SIMPLEC";
    }
}

bool ini_read(const std::string &path, ns3d_params &p, IniFiles &files, std::string &log) {
    std::ifstream in(path.c_str());
    if (!in.is_open()) {
        log += "error: cannot open input file '" + path + "'\n";
        return false;
    }
    ns3d_params_default(&p);
    files = IniFiles();
    bool has_image = false;
    std::string method = "SIMPLEC", precision = "FP64";
    std::string line;
    size_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        line = trim(line);
        if (line.empty() || line[0] == '#') continue;
        size_t eq = line.find('=');
        if (eq == std::string::npos) {
            log += "warning: " + path + ":" + std::to_string(lineno) + " - line ignored (no '=' found)\n";
            continue;
        }
        std::string key = lower(trim(line.substr(0, eq)));
        std::string value = strip_comment(line.substr(eq + 1));
        auto bad = [&](const char *what) {
            log += "error: " + path + ":" + std::to_string(lineno) + " - key '" + key + "' expects a " + what +
                   ", got '" + value + "'\n";
            return false;
        };
        struct DKey { const char *k; double *v; };
        struct IKey { const char *k; int32_t *v; };
        const DKey dkeys[] = {{"dx", &p.dx}, {"dy", &p.dy}, {"dz", &p.dz}, {"mu", &p.mu}, {"rho", &p.rho},
                              {"p0", &p.p0}, {"gradp", &p.gradp}, {"alpha", &p.alpha}, {"beta", &p.beta},
                              {"vsolvertol", &p.vsolvertol}, {"psolvertol", &p.psolvertol},
                              {"pcsolvertol", &p.pcsolvertol}, {"simpletol", &p.simpletol},
                              {"deltaRMR", &p.deltaRMR}};
        const IKey ikeys[] = {{"maxitsolver", &p.maxitsolver}, {"maxitsimple", &p.maxitSIMPLE}, {"n1", &p.N1},
                              {"n2", &p.N2}, {"save_step", &p.save_step}, {"porevalue", &p.porevalue},
                              {"direction", &p.direction}, {"border", &p.border}};
        bool matched = false;
        if (key == "input") { files.input = value; has_image = true; matched = true; }
        else if (key == "pressurefield") { files.pressurefield = value; matched = true; }
        else if (key == "vxfield") { files.vxfield = value; matched = true; }
        else if (key == "vyfield") { files.vyfield = value; matched = true; }
        else if (key == "vzfield") { files.vzfield = value; matched = true; }
        else if (key == "method") { method = value; matched = true; }
        else if (key == "precision") { precision = value; matched = true; }
        if (!matched)
            for (const DKey &d : dkeys)
                if (key == d.k) {
                    double tmp;
                    if (!parse_double(value, tmp)) return bad("number");
                    *d.v = tmp;
                    matched = true;
                    break;
                }
        if (!matched)
            for (const IKey &d : ikeys)
                if (key == d.k) {
                    int tmp;
                    if (!parse_int(value, tmp)) return bad("integer");
                    *d.v = tmp;
                    matched = true;
                    break;
                }
        if (!matched) log += "warning: " + path + ":" + std::to_string(lineno) + " - unknown key '" + key + "' (ignored)\n";
    }
    auto fatal = [&](const std::string &m) {
        log += "error: " + path + " - " + m + "\n";
        return false;
    };
    if (!has_image) return fatal("required key 'input' (image file) is missing");
    if (files.input.empty()) return fatal("key 'input' has an empty value");
    if (p.dx <= 0.0) return fatal("'dx' must be > 0");
    if (p.mu <= 0.0) return fatal("'mu' must be > 0");
    if (p.rho <= 0.0) return fatal("'rho' must be > 0");
    if (p.maxitsolver <= 0) return fatal("'maxitsolver' must be > 0");
    if (p.maxitSIMPLE <= 0) return fatal("'maxitSIMPLE' must be > 0");
    if (p.save_step <= 0) return fatal("'save_step' must be > 0");
    if (p.porevalue != 0 && p.porevalue != 1) {
        log += "warning: " + path + " - 'porevalue' should be 0 or 1, treating '" + std::to_string(p.porevalue) +
               "' as 0\n";
        p.porevalue = 0;
    }
    if (p.direction < 1 || p.direction > 3) return fatal("'direction' must be 1 (x), 2 (y) or 3 (z)");
    std::string m = lower(method);
    if (m == "simplec") p.method = NS3D_SIMPLEC;
    else if (m == "simpler") p.method = NS3D_SIMPLER;
    else if (m == "simplerr") p.method = NS3D_SIMPLERR;
    else if (m == "ideal") p.method = NS3D_IDEAL;
    else return fatal("unknown method '" + method + "'. Valid values: SIMPLEC, SIMPLER, SIMPLERR, IDEAL");
    std::string pr = upper(precision);
    if (pr == "FP64") p.precision = NS3D_FP64;
    else if (pr == "MIXED") p.precision = NS3D_MIXED;
    else if (pr == "MIXED_MG") p.precision = NS3D_MIXED_MG;
    else return fatal("unknown precision '" + precision + "'. Valid values: FP64, MIXED, MIXED_MG");
    if (p.dy <= 0.0) p.dy = p.dx;
    if (p.dz <= 0.0) p.dz = p.dx;
    return true;
}

// ============================ base64 =======================================
static const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

static void b64_encode(const uint8_t *d, size_t n, std::string &out) {
    size_t i = 0;
    for (; i + 2 < n; i += 3) {
        uint32_t v = ((uint32_t)d[i] << 16) | ((uint32_t)d[i + 1] << 8) | d[i + 2];
        out += kB64[(v >> 18) & 63]; out += kB64[(v >> 12) & 63]; out += kB64[(v >> 6) & 63]; out += kB64[v & 63];
    }
    if (i < n) {
        uint32_t v = (uint32_t)d[i] << 16;
        if (i + 1 < n) v |= (uint32_t)d[i + 1] << 8;
        out += kB64[(v >> 18) & 63];
        out += kB64[(v >> 12) & 63];
        out += (i + 1 < n) ? kB64[(v >> 6) & 63] : '=';
        out += '=';
    }
}

static int b64_val(char c) {
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    return -1;
}

// decodes `nchars` base64 characters starting at s (whitespace skipped);
// returns the number of characters consumed (including padding)
static size_t b64_decode(const char *s, size_t avail, size_t want_bytes, std::vector<uint8_t> &out) {
    size_t i = 0;
    uint32_t acc = 0;
    int bits = 0;
    size_t start = out.size();
    while (i < avail && out.size() - start < want_bytes) {
        char c = s[i++];
        if (c == '=') continue;
        int v = b64_val(c);
        if (v < 0) continue;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)((acc >> bits) & 0xff));
        }
    }
    // swallow the padding of this group
    while (i < avail && s[i] == '=') ++i;
    return i;
}

// ============================ .vti reader ===================================
static std::string attr(const std::string &tag, const char *name) {
    std::string key = std::string(" ") + name + "=\"";
    size_t p = tag.find(key);
    if (p == std::string::npos) return std::string();
    p += key.size();
    size_t e = tag.find('"', p);
    return tag.substr(p, e - p);
}

static int type_size(const std::string &t) {
    if (t == "UInt8" || t == "Int8" || t == "unsigned_char" || t == "char") return 1;
    if (t == "UInt16" || t == "Int16" || t == "unsigned_short" || t == "short") return 2;
    if (t == "UInt32" || t == "Int32" || t == "Float32" || t == "unsigned_int" || t == "int" || t == "float") return 4;
    if (t == "UInt64" || t == "Int64" || t == "Float64" || t == "double" || t == "unsigned_long" || t == "long") return 8;
    return 0;
}

static bool read_file(const std::string &path, std::string &buf) {
    std::ifstream in(path.c_str(), std::ios::binary);
    if (!in) return false;
    std::ostringstream ss;
    ss << in.rdbuf();
    buf = ss.str();
    return true;
}

// one binary block: [header][payload], header = nbytes (uncompressed) or
// [nblocks, blocksize, lastsize, csize_1..csize_n] (compressed)
static bool decode_block(const char *s, size_t avail, bool is_b64, bool compressed, int hsize, size_t nbytes,
                         std::vector<uint8_t> &out, std::string &err) {
    auto rd = [&](const uint8_t *p) -> uint64_t {
        if (hsize == 4) { uint32_t v; std::memcpy(&v, p, 4); return v; }
        uint64_t v; std::memcpy(&v, p, 8); return v;
    };
    out.clear();
    if (!compressed) {
        std::vector<uint8_t> all;
        if (is_b64) {
            // the header may be encoded on its own (padded) or with the data
            size_t hchars = ((size_t)hsize + 2) / 3 * 4;
            bool separate = hchars <= avail && std::memchr(s, '=', hchars) != nullptr;
            if (separate) {
                std::vector<uint8_t> h;
                size_t used = b64_decode(s, avail, (size_t)hsize, h);
                b64_decode(s + used, avail - used, nbytes, all);
            } else {
                b64_decode(s, avail, (size_t)hsize + nbytes, all);
                if (all.size() >= (size_t)hsize) all.erase(all.begin(), all.begin() + hsize);
            }
        } else {
            if (avail < (size_t)hsize + nbytes) { err = "truncated raw data"; return false; }
            all.assign((const uint8_t *)s + hsize, (const uint8_t *)s + hsize + nbytes);
        }
        if (all.size() < nbytes) { err = "truncated data array"; return false; }
        all.resize(nbytes);
        out.swap(all);
        return true;
    }
    // compressed
    std::vector<uint8_t> h;
    size_t used = 0;
    const uint8_t *hp;
    std::vector<uint8_t> first;
    if (is_b64) {
        size_t c3 = b64_decode(s, avail, (size_t)hsize * 3, first);
        (void)c3;
        if (first.size() < (size_t)hsize * 3) { err = "truncated header"; return false; }
        uint64_t nb = rd(first.data());
        size_t hlen = (size_t)(3 + nb) * hsize;
        used = b64_decode(s, avail, hlen, h);
        if (h.size() < hlen) { err = "truncated header"; return false; }
        hp = h.data();
    } else {
        if (avail < (size_t)hsize * 3) { err = "truncated header"; return false; }
        uint64_t nb = rd((const uint8_t *)s);
        size_t hlen = (size_t)(3 + nb) * hsize;
        if (avail < hlen) { err = "truncated header"; return false; }
        h.assign((const uint8_t *)s, (const uint8_t *)s + hlen);
        hp = h.data();
        used = hlen;
    }
    uint64_t nblocks = rd(hp), bsize = rd(hp + hsize), last = rd(hp + 2 * hsize);
    std::vector<uint64_t> cs(nblocks);
    uint64_t total = 0;
    for (uint64_t b = 0; b < nblocks; ++b) { cs[b] = rd(hp + (3 + b) * hsize); total += cs[b]; }
    std::vector<uint8_t> comp;
    if (is_b64) {
        b64_decode(s + used, avail - used, (size_t)total, comp);
    } else {
        if (avail - used < total) { err = "truncated compressed data"; return false; }
        comp.assign((const uint8_t *)s + used, (const uint8_t *)s + used + total);
    }
    if (comp.size() < total) { err = "truncated compressed data"; return false; }
    out.reserve((size_t)(bsize * nblocks));
    size_t pos = 0;
    for (uint64_t b = 0; b < nblocks; ++b) {
        uLongf dl = (uLongf)((b + 1 == nblocks && last != 0) ? last : bsize);
        std::vector<uint8_t> tmp(dl);
        int zr = uncompress(tmp.data(), &dl, comp.data() + pos, (uLong)cs[b]);
        if (zr != Z_OK) { err = "zlib error " + std::to_string(zr); return false; }
        out.insert(out.end(), tmp.begin(), tmp.begin() + dl);
        pos += cs[b];
    }
    if (out.size() < nbytes) { err = "decompressed size mismatch"; return false; }
    out.resize(nbytes);
    return true;
}

// legacy .vtk STRUCTURED_POINTS (vtkStructuredPointsReader): BINARY data is big endian
static bool vtk_legacy_read(const std::string &buf, VtiImage &img, std::string &err) {
    size_t pos = 0;
    auto next_line = [&](std::string &l) {
        if (pos >= buf.size()) return false;
        size_t e = buf.find('\n', pos);
        if (e == std::string::npos) e = buf.size();
        l = buf.substr(pos, e - pos);
        if (!l.empty() && l.back() == '\r') l.pop_back();
        pos = e + 1;
        return true;
    };
    std::string l;
    next_line(l);  // version
    next_line(l);  // title
    next_line(l);
    bool binary = upper(trim(l)) == "BINARY";
    std::string type;
    int ncomp = 1;
    while (next_line(l)) {
        std::istringstream ls(l);
        std::string kw;
        ls >> kw;
        kw = upper(kw);
        if (kw == "DIMENSIONS") ls >> img.dims[0] >> img.dims[1] >> img.dims[2];
        else if (kw == "SCALARS") {
            std::string name;
            ls >> name >> type;
            if (!(ls >> ncomp)) ncomp = 1;
        } else if (kw == "LOOKUP_TABLE") break;
    }
    int ts = type_size(type);
    if (ts == 0 || img.dims[0] <= 0) { err = "unsupported legacy .vtk content"; return false; }
    img.ncomp = ncomp;
    img.type = type == "unsigned_char" ? "UInt8" : type == "char" ? "Int8" : type == "float" ? "Float32"
             : type == "double" ? "Float64" : type == "int" ? "Int32" : type == "short" ? "Int16"
             : type == "unsigned_short" ? "UInt16" : type;
    size_t n = (size_t)img.dims[0] * img.dims[1] * img.dims[2] * ncomp;
    img.raw.resize(n * ts);
    if (binary) {
        if (buf.size() - pos < n * ts) { err = "truncated legacy .vtk data"; return false; }
        for (size_t i = 0; i < n; ++i)
            for (int b = 0; b < ts; ++b) img.raw[i * ts + b] = (uint8_t)buf[pos + i * ts + (ts - 1 - b)];
    } else {
        std::istringstream ds(buf.substr(pos));
        for (size_t i = 0; i < n; ++i) {
            double v;
            if (!(ds >> v)) { err = "truncated legacy .vtk data"; return false; }
            if (ts == 1) img.raw[i] = (uint8_t)(int)v;
            else if (img.type == "Float32") { float f = (float)v; std::memcpy(&img.raw[i * 4], &f, 4); }
            else if (img.type == "Float64") std::memcpy(&img.raw[i * 8], &v, 8);
            else { err = "unsupported ascii legacy type"; return false; }
        }
    }
    return true;
}

bool vti_read(const std::string &path, VtiImage &img, std::string &err) {
    std::string buf;
    if (!read_file(path, buf)) { err = "cannot open " + path; return false; }
    if (path.size() >= 3 && path.substr(path.size() - 3) == "vtk") return vtk_legacy_read(buf, img, err);
    size_t vt = buf.find("<VTKFile");
    if (vt == std::string::npos) { err = "not a VTK XML file: " + path; return false; }
    std::string vtag = buf.substr(vt, buf.find('>', vt) - vt);
    if (attr(vtag, "byte_order") == "BigEndian") { err = "big-endian .vti is not supported"; return false; }
    int hsize = attr(vtag, "header_type") == "UInt64" ? 8 : 4;
    bool compressed = !attr(vtag, "compressor").empty();
    size_t it = buf.find("<ImageData");
    if (it == std::string::npos) { err = "no ImageData element"; return false; }
    std::string itag = buf.substr(it, buf.find('>', it) - it);
    int e[6];
    if (sscanf(attr(itag, "WholeExtent").c_str(), "%d %d %d %d %d %d", e, e + 1, e + 2, e + 3, e + 4, e + 5) != 6) {
        err = "bad WholeExtent";
        return false;
    }
    img.dims[0] = e[1] - e[0] + 1;
    img.dims[1] = e[3] - e[2] + 1;
    img.dims[2] = e[5] - e[4] + 1;
    size_t da = buf.find("<DataArray", it);
    if (da == std::string::npos) { err = "no DataArray"; return false; }
    size_t daend = buf.find('>', da);
    std::string dtag = buf.substr(da, daend - da);
    img.type = attr(dtag, "type");
    std::string nc = attr(dtag, "NumberOfComponents");
    img.ncomp = nc.empty() ? 1 : std::atoi(nc.c_str());
    int ts = type_size(img.type);
    if (ts == 0) { err = "unsupported data type " + img.type; return false; }
    size_t nbytes = (size_t)img.dims[0] * img.dims[1] * img.dims[2] * img.ncomp * ts;
    std::string fmt = attr(dtag, "format");
    if (fmt == "appended") {
        size_t ad = buf.find("<AppendedData", daend);
        if (ad == std::string::npos) { err = "no AppendedData"; return false; }
        std::string atag = buf.substr(ad, buf.find('>', ad) - ad);
        bool b64 = attr(atag, "encoding") != "raw";
        size_t us = buf.find('_', ad);
        if (us == std::string::npos) { err = "no appended data marker"; return false; }
        size_t off = (size_t)std::atoll(attr(dtag, "offset").c_str());
        size_t start = us + 1 + off;
        if (start > buf.size()) { err = "bad offset"; return false; }
        return decode_block(buf.data() + start, buf.size() - start, b64, compressed, hsize, nbytes, img.raw, err);
    } else if (fmt == "binary") {
        size_t start = daend + 1;
        size_t stop = buf.find("</DataArray>", start);
        return decode_block(buf.data() + start, stop - start, true, compressed, hsize, nbytes, img.raw, err);
    } else if (fmt == "ascii") {
        size_t start = daend + 1;
        std::istringstream ds(buf.substr(start, buf.find("</DataArray>", start) - start));
        size_t n = nbytes / ts;
        img.raw.resize(nbytes);
        for (size_t i = 0; i < n; ++i) {
            double v;
            if (!(ds >> v)) { err = "truncated ascii data"; return false; }
            if (ts == 1) img.raw[i] = (uint8_t)(int)v;
            else if (img.type == "Float32") { float f = (float)v; std::memcpy(&img.raw[i * 4], &f, 4); }
            else if (img.type == "Float64") std::memcpy(&img.raw[i * 8], &v, 8);
            else { err = "unsupported ascii type"; return false; }
        }
        return true;
    }
    err = "unsupported DataArray format '" + fmt + "'";
    return false;
}

bool vti_to_f64(const VtiImage &img, std::vector<double> &out, std::string &err) {
    size_t n = (size_t)img.dims[0] * img.dims[1] * img.dims[2] * img.ncomp;
    out.resize(n);
    const uint8_t *p = img.raw.data();
    const std::string &t = img.type;
    for (size_t i = 0; i < n; ++i) {
        if (t == "Float64") std::memcpy(&out[i], p + 8 * i, 8);
        else if (t == "Float32") { float f; std::memcpy(&f, p + 4 * i, 4); out[i] = f; }
        else if (t == "UInt8") out[i] = p[i];
        else if (t == "Int8") out[i] = (int8_t)p[i];
        else if (t == "Int32") { int32_t v; std::memcpy(&v, p + 4 * i, 4); out[i] = v; }
        else if (t == "UInt32") { uint32_t v; std::memcpy(&v, p + 4 * i, 4); out[i] = v; }
        else if (t == "Int16") { int16_t v; std::memcpy(&v, p + 2 * i, 2); out[i] = v; }
        else if (t == "UInt16") { uint16_t v; std::memcpy(&v, p + 2 * i, 2); out[i] = v; }
        else { err = "cannot convert " + t; return false; }
    }
    return true;
}

// ============================ .vti writer ===================================
static bool write_vti(const std::string &path, const char *type, const uint8_t *data, size_t nbytes, int nx, int ny,
                      int nz, int ncomp, double rmin, double rmax, std::string &err) {
    const size_t bs = 32768;
    size_t nblocks = (nbytes + bs - 1) / bs;
    size_t last = nbytes % bs;
    std::vector<uint32_t> hdr(3 + nblocks);
    hdr[0] = (uint32_t)nblocks;
    hdr[1] = (uint32_t)bs;
    hdr[2] = (uint32_t)last;
    std::vector<uint8_t> comp;
    comp.reserve(nbytes / 4 + 1024);
    for (size_t b = 0; b < nblocks; ++b) {
        size_t len = std::min(bs, nbytes - b * bs);
        uLongf cl = compressBound((uLong)len);
        std::vector<uint8_t> tmp(cl);
        if (compress2(tmp.data(), &cl, data + b * bs, (uLong)len, 5) != Z_OK) { err = "zlib compress failed"; return false; }
        hdr[3 + b] = (uint32_t)cl;
        comp.insert(comp.end(), tmp.begin(), tmp.begin() + cl);
    }
    std::string enc;
    b64_encode((const uint8_t *)hdr.data(), hdr.size() * 4, enc);
    b64_encode(comp.data(), comp.size(), enc);
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { err = "cannot write " + path; return false; }
    fprintf(f, "<?xml version=\"1.0\"?>\n");
    fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt32\" "
               "compressor=\"vtkZLibDataCompressor\">\n");
    fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"0 0 0\" Spacing=\"1 1 1\" "
               "Direction=\"1 0 0 0 1 0 0 0 1\">\n", nx - 1, ny - 1, nz - 1);
    fprintf(f, "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", nx - 1, ny - 1, nz - 1);
    if (ncomp == 1) fprintf(f, "      <PointData Scalars=\"ImageScalars\">\n");
    else fprintf(f, "      <PointData Scalars=\"ImageScalars\">\n");
    fprintf(f, "        <DataArray type=\"%s\" Name=\"ImageScalars\"", type);
    if (ncomp > 1) fprintf(f, " NumberOfComponents=\"%d\"", ncomp);
    fprintf(f, " format=\"appended\" RangeMin=\"%.11g\" RangeMax=\"%.11g\" offset=\"0\" />\n", rmin, rmax);
    fprintf(f, "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n");
    fprintf(f, "  <AppendedData encoding=\"base64\">\n   _");
    fwrite(enc.data(), 1, enc.size(), f);
    fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
    bool ok = fclose(f) == 0;
    if (!ok) err = "write error " + path;
    return ok;
}

bool vti_write_f64(const std::string &path, const double *data, int nx, int ny, int nz, int ncomp, std::string &err) {
    size_t n = (size_t)nx * ny * nz;
    std::vector<double> xf(n * ncomp);
    double rmin = 0, rmax = 0;
    bool first = true;
    // C order (x slowest) -> VTK order (x fastest)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                for (int c = 0; c < ncomp; ++c) {
                    double v = data[(((size_t)i * ny + j) * nz + k) * ncomp + c];
                    xf[(((size_t)k * ny + j) * nx + i) * ncomp + c] = v;
                    if (first || v < rmin) rmin = v;
                    if (first || v > rmax) rmax = v;
                    first = false;
                }
    return write_vti(path, "Float64", (const uint8_t *)xf.data(), xf.size() * 8, nx, ny, nz, ncomp, rmin, rmax, err);
}

bool vti_write_u8(const std::string &path, const uint8_t *data, int nx, int ny, int nz, std::string &err) {
    size_t n = (size_t)nx * ny * nz;
    double rmin = 255, rmax = 0;
    for (size_t i = 0; i < n; ++i) {
        rmin = std::min<double>(rmin, data[i]);
        rmax = std::max<double>(rmax, data[i]);
    }
    return write_vti(path, "UInt8", data, n, nx, ny, nz, 1, rmin, rmax, err);
}

}  // namespace ns3d
