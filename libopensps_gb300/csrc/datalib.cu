// The standard-format data reader (host code): a small JSON parser, the library/manifest checks and raw array reads
// of src/io/opensps_datalib.f90, and the per-kind processing onto the model's wavelength grid of the readers in
// src/io/opensps_io.f90 and src/spectra/opensps_filters.f90 that this path uses.
#include "datalib.h"

#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "context.h"
#include "csp_kernels.h"

namespace sps {

// ---------------------------------------------------------------------------------------------- JSON
const JVal *JVal::get(const std::string &k) const {
    if (kind != OBJ) return nullptr;
    for (size_t i = 0; i < keys.size(); ++i)
        if (keys[i] == k) return &items[i];
    return nullptr;
}

namespace {
struct JParser {
    const std::string &s;
    size_t p = 0;
    std::string err;
    explicit JParser(const std::string &t) : s(t) {}
    void ws() { while (p < s.size() && (s[p] == ' ' || s[p] == '\t' || s[p] == '\n' || s[p] == '\r')) ++p; }
    bool fail(const char *m) { if (err.empty()) err = std::string(m) + " at offset " + std::to_string(p); return false; }
    static void utf8(std::string &o, unsigned cp) {
        if (cp < 0x80) o += (char)cp;
        else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
        else if (cp < 0x10000) { o += (char)(0xE0 | (cp >> 12)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
        else { o += (char)(0xF0 | (cp >> 18)); o += (char)(0x80 | ((cp >> 12) & 0x3F)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
    }
    bool hex4(unsigned &v) {
        if (p + 4 > s.size()) return fail("short \\u escape");
        v = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = s[p++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool str(std::string &o) {
        if (p >= s.size() || s[p] != '"') return fail("expected a string");
        ++p;
        while (p < s.size() && s[p] != '"') {
            const unsigned char c = (unsigned char)s[p++];
            if (c < 0x20) return fail("control character in a string");
            if (c != '\\') { o += (char)c; continue; }
            if (p >= s.size()) return fail("unterminated escape");
            const char e = s[p++];
            switch (e) {
                case '"': o += '"'; break;
                case '\\': o += '\\'; break;
                case '/': o += '/'; break;
                case 'b': o += '\b'; break;
                case 'f': o += '\f'; break;
                case 'n': o += '\n'; break;
                case 'r': o += '\r'; break;
                case 't': o += '\t'; break;
                case 'u': {
                    unsigned cp;
                    if (!hex4(cp)) return false;
                    if (cp >= 0xD800 && cp < 0xDC00 && p + 6 <= s.size() && s[p] == '\\' && s[p + 1] == 'u') {
                        p += 2;
                        unsigned lo;
                        if (!hex4(lo)) return false;
                        if (lo < 0xDC00 || lo >= 0xE000) return fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(o, cp);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        if (p >= s.size()) return fail("unterminated string");
        ++p;
        return true;
    }
    bool num(JVal &v) {
        const size_t b = p;
        if (p < s.size() && s[p] == '-') ++p;
        if (p >= s.size() || !std::isdigit((unsigned char)s[p])) return fail("bad number");
        if (s[p] == '0') ++p;
        else while (p < s.size() && std::isdigit((unsigned char)s[p])) ++p;
        if (p < s.size() && s[p] == '.') {
            ++p;
            if (p >= s.size() || !std::isdigit((unsigned char)s[p])) return fail("bad number");
            while (p < s.size() && std::isdigit((unsigned char)s[p])) ++p;
        }
        if (p < s.size() && (s[p] == 'e' || s[p] == 'E')) {
            ++p;
            if (p < s.size() && (s[p] == '+' || s[p] == '-')) ++p;
            if (p >= s.size() || !std::isdigit((unsigned char)s[p])) return fail("bad number");
            while (p < s.size() && std::isdigit((unsigned char)s[p])) ++p;
        }
        v.kind = JVal::NUM;
        v.num = std::strtod(s.substr(b, p - b).c_str(), nullptr);   // correctly rounded (C locale)
        return true;
    }
    bool lit(const char *w, JVal &v, JVal::Kind k, bool bv) {
        const size_t n = std::strlen(w);
        if (s.compare(p, n, w) != 0) return fail("bad literal");
        p += n;
        v.kind = k;
        v.b = bv;
        return true;
    }
    bool value(JVal &v, int depth) {
        if (depth > 256) return fail("nesting too deep");
        ws();
        if (p >= s.size()) return fail("unexpected end");
        const char c = s[p];
        if (c == '{') {
            ++p;
            v.kind = JVal::OBJ;
            ws();
            if (p < s.size() && s[p] == '}') { ++p; return true; }
            for (;;) {
                ws();
                std::string k;
                if (!str(k)) return false;
                ws();
                if (p >= s.size() || s[p] != ':') return fail("expected ':'");
                ++p;
                JVal item;
                if (!value(item, depth + 1)) return false;
                v.keys.push_back(k);
                v.items.push_back(std::move(item));
                ws();
                if (p < s.size() && s[p] == ',') { ++p; continue; }
                if (p < s.size() && s[p] == '}') { ++p; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p;
            v.kind = JVal::ARR;
            ws();
            if (p < s.size() && s[p] == ']') { ++p; return true; }
            for (;;) {
                JVal item;
                if (!value(item, depth + 1)) return false;
                v.items.push_back(std::move(item));
                ws();
                if (p < s.size() && s[p] == ',') { ++p; continue; }
                if (p < s.size() && s[p] == ']') { ++p; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') { v.kind = JVal::STR; return str(v.str); }
        if (c == 't') return lit("true", v, JVal::BOOL, true);
        if (c == 'f') return lit("false", v, JVal::BOOL, false);
        if (c == 'n') return lit("null", v, JVal::NUL, false);
        return num(v);
    }
};

bool read_text(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

bool file_exists(const std::string &path) {
    struct stat st;
    return ::stat(path.c_str(), &st) == 0;
}

std::string base_name(const std::string &spec) {
    const size_t k = spec.find(':');
    std::string n = k == std::string::npos ? spec : spec.substr(0, k);
    while (!n.empty() && n.back() == ' ') n.pop_back();
    return n;
}

std::string lower(std::string s) {
    for (char &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// trapezoid integral with |dx| (integrate_trapezoid_array, src/math/opensps_integration.f90:68-92)
double trapz_abs(const double *x, const double *y, int n) {
    double s = 0.0;
    for (int i = 0; i + 1 < n; ++i) s += std::fabs(x[i + 1] - x[i]) * (y[i + 1] + y[i]);
    return 0.5 * s;
}

// interpolate_linear_scalar (src/math/opensps_interpolation.f90:45-72): the bracketing interval clamped to the
// table, linear (so extrapolated) beyond it
int bad(std::string &err, const std::string &msg, int st = ST_DATA_MISSING) {
    err = msg;
    return st;
}

double interp_linear(const double *x, const double *y, int n, double v) {
    int i = find_interval0(x, n, v);
    i = std::max(0, std::min(i, n - 2));
    const double slope = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
    return y[i] + slope * (v - x[i]);
}
}  // namespace

bool json_parse(const std::string &text, JVal &out, std::string &err) {
    JParser ps(text);
    out = JVal();
    if (!ps.value(out, 0)) { err = ps.err; return false; }
    ps.ws();
    if (ps.p != text.size()) { err = "trailing characters at offset " + std::to_string(ps.p); return false; }
    return true;
}

// ---------------------------------------------------------------------------------------------- format selection
DataFormat data_format_from_env() {
    const char *e = std::getenv("OPENSPS_DATA_FORMAT");
    if (!e || !*e) e = std::getenv("FSPS_DATA_FORMAT");
    if (!e || !*e) return DF_AUTO;
    const std::string v = lower(trim(e));
    if (v == "legacy") return DF_LEGACY;
    if (v == "standard" || v == "std") return DF_STANDARD;
    if (v == "auto" || v.empty()) return DF_AUTO;
    return DF_BAD;
}

bool datalib_root_is_standard(const std::string &root) {
    return file_exists(root + "/opensps-data.json") || file_exists(root + "/fsps-data.json");
}

bool datalib_available(const std::string &root, const std::string &kind, const std::string &name) {
    switch (data_format_from_env()) {
        case DF_LEGACY: return false;
        case DF_STANDARD: return true;
        default: return file_exists(root + "/libraries/" + kind + "/" + base_name(name) + "/manifest.json");
    }
}

// ---------------------------------------------------------------------------------------------- libraries
int DataLib::fail(std::string &err, const std::string &msg) const {
    err = "library " + kind + "/" + name + " (" + dir + "): " + msg;
    return ST_DATA_MISSING;
}

int DataLib::open(const std::string &root, const std::string &k, const std::string &spec, std::string &err) {
    kind = k;
    name = base_name(spec);
    dir = root + "/libraries/" + kind + "/" + name;
    sel.clear();
    std::string text, jerr;
    if (!read_text(dir + "/manifest.json", text)) {
        err = "cannot read the manifest of library " + kind + "/" + name + " under " + dir +
              (datalib_root_is_standard(root) ? "" : " (" + root + " has no opensps-data.json: not a standard-format data root)");
        return ST_DATA_MISSING;
    }
    if (!json_parse(text, doc, jerr)) return fail(err, "manifest.json: " + jerr);
    if (doc.kind != JVal::OBJ) return fail(err, "manifest.json is not a JSON object");
    const JVal *f = doc.get("format");
    if (!f || f->kind != JVal::STR || (f->str != "opensps-data" && f->str != "fsps-data"))
        return fail(err, "manifest.json is not an opensps-data manifest (field \"format\")");
    const JVal *v = doc.get("format_version");
    if (!v || v->kind != JVal::NUM || v->num != 1.0) return fail(err, "unsupported format_version (this code reads version 1)");
    const JVal *kd = doc.get("kind");
    if (!kd || kd->kind != JVal::STR || kd->str != kind)
        return fail(err, "manifest kind is \"" + (kd && kd->kind == JVal::STR ? kd->str : std::string()) + "\", expected \"" + kind + "\"");
    const JVal *nm = doc.get("name");
    if (!nm || nm->kind != JVal::STR || nm->str != name) return fail(err, "manifest name differs from the directory name");
    const JVal *ax = doc.get("axes"), *ar = doc.get("arrays");
    if (!ax || ax->kind != JVal::OBJ) return fail(err, "missing \"axes\" object");
    if (!ar || ar->kind != JVal::OBJ) return fail(err, "missing \"arrays\" object");
    // axis selections after ':'
    const size_t c = spec.find(':');
    if (c != std::string::npos) {
        std::stringstream ss(spec.substr(c + 1));
        std::string item;
        while (std::getline(ss, item, ',')) {
            item = trim(item);
            if (item.empty()) continue;
            const size_t e = item.find('=');
            if (e == std::string::npos || e == 0) return fail(err, "bad axis selection \"" + item + "\" (expected axis=value)");
            if (sel.size() == 8) return fail(err, "too many axis selections");
            const std::string a = trim(item.substr(0, e)), val = trim(item.substr(e + 1));
            if (!has_axis(a)) return fail(err, "selection on unknown axis \"" + a + "\"");
            sel.emplace_back(a, val);
        }
    }
    return 0;
}

const JVal *DataLib::meta(const std::string &key) const {
    const JVal *m = doc.get("metadata");
    return m ? m->get(key) : nullptr;
}
bool DataLib::has_axis(const std::string &axis) const { return doc.get("axes")->get(axis) != nullptr; }
bool DataLib::has_array(const std::string &n) const { return doc.get("arrays")->get(n) != nullptr; }

static bool shape_of(const JVal &d, std::vector<long long> &dims) {
    const JVal *s = d.get("shape");
    if (!s || s->kind != JVal::ARR || s->items.empty()) return false;
    dims.clear();
    for (const JVal &x : s->items) {
        if (x.kind != JVal::NUM || x.num < 0 || x.num != std::floor(x.num)) return false;
        dims.push_back((long long)x.num);
    }
    return true;
}

int DataLib::axis_len(const std::string &axis, long long &n, std::string &err) const {
    const JVal *a = doc.get("axes")->get(axis);
    if (!a) return fail(err, "no axis \"" + axis + "\"");
    if (const JVal *l = a->get("labels")) { n = (long long)l->items.size(); return 0; }
    if (const JVal *v = a->get("values")) { n = (long long)v->items.size(); return 0; }
    std::vector<long long> dims;
    if (!shape_of(*a, dims)) return fail(err, "axis " + axis + ": \"shape\" must be a list of integers");
    if (dims.size() != 1) return fail(err, "axis \"" + axis + "\" must be one-dimensional");
    n = dims[0];
    return 0;
}

int DataLib::axis_values(const std::string &axis, std::vector<double> &vals, std::string &err) const {
    const JVal *a = doc.get("axes")->get(axis);
    if (!a) return fail(err, "no axis \"" + axis + "\"");
    if (const JVal *v = a->get("values")) {
        vals.clear();
        for (const JVal &x : v->items) {
            if (x.kind != JVal::NUM) return fail(err, "axis \"" + axis + "\": values must be numbers");
            vals.push_back(x.num);
        }
        return 0;
    }
    if (a->get("file")) {
        long long n = 0;
        if (int rc = axis_len(axis, n, err)) return rc;
        return read_desc(*a, "axis " + axis, n, 0, false, &vals, nullptr, err);
    }
    return fail(err, "axis \"" + axis + "\" has no numeric coordinates");
}

int DataLib::array_len(const std::string &n, long long &len, std::string &err) const {
    const JVal *d = doc.get("arrays")->get(n);
    if (!d) return fail(err, "no array \"" + n + "\"");
    std::vector<long long> dims;
    if (!shape_of(*d, dims)) return fail(err, "array " + n + ": \"shape\" must be a list of integers");
    len = 1;
    for (long long x : dims) len *= x;
    return 0;
}

int DataLib::select_index(const std::string &axis, const std::string &value, int &idx, std::string &err) const {
    idx = -1;
    const JVal *a = doc.get("axes")->get(axis);
    if (const JVal *l = a->get("labels")) {
        for (size_t i = 0; i < l->items.size(); ++i)
            if (l->items[i].kind == JVal::STR && l->items[i].str == value) idx = (int)i;
    } else {
        char *end = nullptr;
        const double v = std::strtod(value.c_str(), &end);
        if (end == value.c_str() || *end != '\0') return fail(err, "selection \"" + axis + "=" + value + "\" is not a number");
        std::vector<double> vals;
        if (int rc = axis_values(axis, vals, err)) return rc;
        for (size_t i = 0; i < vals.size(); ++i)
            if (std::fabs(vals[i] - v) <= 1.0e-9 * std::max(1.0, std::fabs(v))) idx = (int)i;
    }
    if (idx < 0) return fail(err, "axis \"" + axis + "\" has no value " + value);
    return 0;
}

int DataLib::check_array(const std::string &n, const std::vector<std::string> &axes, const std::vector<long long> &dims,
                         long long &offset, std::string &err) const {
    const JVal *d = doc.get("arrays")->get(n);
    if (!d) return fail(err, "no array \"" + n + "\"");
    std::vector<long long> shp;
    if (!shape_of(*d, shp)) return fail(err, "array " + n + ": \"shape\" must be a list of integers");
    const JVal *an = d->get("axes");
    const size_t nax = shp.size(), nreq = axes.size();
    if (!an || an->kind != JVal::ARR || an->items.size() != nax)
        return fail(err, "array \"" + n + "\": \"axes\" must name each of its dimensions");
    for (const JVal &x : an->items)
        if (x.kind != JVal::STR) return fail(err, "array \"" + n + "\": \"axes\" must be names");
    if (nax < nreq) return fail(err, "array \"" + n + "\" has fewer dimensions than its kind requires");
    const size_t nextra = nax - nreq;
    for (size_t i = 0; i < nreq; ++i) {
        const std::string &axn = an->items[nextra + i].str;
        if (axn != axes[i])
            return fail(err, "array \"" + n + "\": dimension " + std::to_string(nextra + i + 1) + " is \"" + axn +
                                 "\", expected \"" + axes[i] + "\"");
        if (shp[nextra + i] != dims[i])
            return fail(err, "array \"" + n + "\": axis \"" + axn + "\" has " + std::to_string(shp[nextra + i]) +
                                 " entries, expected " + std::to_string(dims[i]));
        long long al = 0;
        if (int rc = axis_len(axn, al, err)) return rc;
        if (al != shp[nextra + i]) return fail(err, "array \"" + n + "\": its dimension differs from the length of axis \"" + axn + "\"");
    }
    // the selected block: C order, the last extra axis varies fastest
    offset = 0;
    long long stride = 1;
    for (long long x : dims) stride *= x;
    for (size_t i = nextra; i-- > 0;) {
        const std::string &axn = an->items[i].str;
        int idx = 0;
        if (shp[i] > 1) {
            idx = -1;
            for (const auto &s : sel)
                if (s.first == axn)
                    if (int rc = select_index(axn, s.second, idx, err)) return rc;
            if (idx < 0) {
                const JVal *ax = doc.get("axes")->get(axn);
                const JVal *df = ax ? ax->get("default") : nullptr;
                if (df && df->kind == JVal::STR) {
                    if (int rc = select_index(axn, df->str, idx, err)) return rc;
                } else if (df && df->kind == JVal::NUM) {
                    char buf[40];
                    std::snprintf(buf, sizeof buf, "%.17g", df->num);
                    if (int rc = select_index(axn, buf, idx, err)) return rc;
                }
            }
            if (idx < 0)
                return fail(err, "array \"" + n + "\" has an extra axis \"" + axn + "\" of length " + std::to_string(shp[i]) +
                                     ": select one value with \"" + name + ":" + axn + "=<value>\"");
        }
        offset += (long long)idx * stride;
        stride *= shp[i];
    }
    return 0;
}

int DataLib::read_desc(const JVal &d, const std::string &what, long long n, long long offset, bool integer,
                       std::vector<double> *outf, std::vector<long long> *outi, std::string &err) const {
    const JVal *dt = d.get("dtype"), *fl = d.get("file");
    const std::string dtype = dt && dt->kind == JVal::STR ? dt->str : std::string();
    const int isz = (dtype == "<f4" || dtype == "<i4") ? 4 : (dtype == "<f8" || dtype == "<i8") ? 8 : 0;
    if (isz == 0) return fail(err, what + ": unsupported dtype \"" + dtype + "\" (use <f4, <f8, <i4 or <i8)");
    if (!fl || fl->kind != JVal::STR) return fail(err, what + ": missing \"file\"");
    const std::string path = dir + "/" + fl->str;
    std::vector<long long> dims;
    if (!shape_of(d, dims)) return fail(err, what + ": \"shape\" must be a list of integers");
    long long total = 1;
    for (long long x : dims) total *= x;
    if (offset < 0 || n < 0 || offset + n > total) return fail(err, what + ": read beyond the array");
    struct stat st;
    if (::stat(path.c_str(), &st) != 0) return fail(err, what + ": file " + path + " is missing");
    if ((long long)st.st_size != total * isz)
        return fail(err, what + ": file " + path + " has " + std::to_string((long long)st.st_size) + " bytes, expected " +
                             std::to_string(total * isz) + " (truncated download?)");
    const bool is_int = dtype[1] == 'i';
    if (is_int != integer)
        return fail(err, integer ? what + " must be an integer array (<i4 or <i8)" : what + " must be a floating-point array (<f4 or <f8)");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(err, what + ": cannot open " + path);
    std::vector<unsigned char> raw((size_t)n * isz);
    f.seekg((std::streamoff)(offset * isz));
    f.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)raw.size());
    if ((size_t)f.gcount() != raw.size()) return fail(err, what + ": short read of " + path);
    // little-endian bytes to host values, byte by byte (independent of the host's order)
    auto u64 = [&](size_t i) {
        uint64_t v = 0;
        for (int b = isz - 1; b >= 0; --b) v = (v << 8) | raw[i * isz + b];
        return v;
    };
    if (integer) {
        outi->resize((size_t)n);
        for (long long i = 0; i < n; ++i) {
            const uint64_t v = u64((size_t)i);
            (*outi)[(size_t)i] = isz == 4 ? (long long)(int32_t)(uint32_t)v : (long long)(int64_t)v;
        }
    } else {
        outf->resize((size_t)n);
        for (long long i = 0; i < n; ++i) {
            const uint64_t v = u64((size_t)i);
            if (isz == 4) {
                const uint32_t w = (uint32_t)v;
                float x;
                std::memcpy(&x, &w, 4);
                (*outf)[(size_t)i] = (double)x;      // FP32 promoted exactly
            } else {
                double x;
                std::memcpy(&x, &v, 8);
                (*outf)[(size_t)i] = x;
            }
        }
    }
    return 0;
}

int DataLib::read_real(const std::string &n, long long cnt, long long offset, std::vector<double> &out, std::string &err) const {
    const JVal *d = doc.get("arrays")->get(n);
    if (!d) return fail(err, "no array \"" + n + "\"");
    return read_desc(*d, "array " + n, cnt, offset, false, &out, nullptr, err);
}

int DataLib::read_int(const std::string &n, long long cnt, long long offset, std::vector<long long> &out, std::string &err) const {
    const JVal *d = doc.get("arrays")->get(n);
    if (!d) return fail(err, "no array \"" + n + "\"");
    return read_desc(*d, "array " + n, cnt, offset, true, nullptr, &out, err);
}

// ---------------------------------------------------------------------------------------------- kinds
int std_load_ssp(const std::string &root, const std::string &spec, SspLibrary &o, std::string &err) {
    DataLib lib;
    if (int rc = lib.open(root, "ssp", spec, err)) return rc;
    const JVal *zs = lib.meta("solar_metallicity");
    if (!zs || zs->kind != JVal::NUM || !(zs->num > 0.0))
        return bad(err, "library ssp/" + lib.name + ": metadata solar_metallicity is required");
    o.zsol = zs->num;
    if (int rc = lib.axis_values("wavelength", o.lam, err)) return rc;
    if (int rc = lib.axis_values("log_age", o.log_age, err)) return rc;
    std::string zax = "Z";
    if (lib.has_axis("Z")) {
        if (int rc = lib.axis_values("Z", o.zlegend, err)) return rc;
    } else if (lib.has_axis("feh")) {
        zax = "feh";
        if (int rc = lib.axis_values("feh", o.zlegend, err)) return rc;
        for (double &z : o.zlegend) z = o.zsol * std::pow(10.0, z);
    } else {
        return bad(err, "library ssp/" + lib.name + ": no metallicity axis (Z or feh)");
    }
    o.nspec = (int)o.lam.size();
    o.nt = (int)o.log_age.size();
    o.nz = (int)o.zlegend.size();
    if (o.nspec < 2 || o.nt < 1 || o.nz < 1) return bad(err, "library ssp/" + lib.name + ": empty grid");
    for (int j = 0; j + 1 < o.nspec; ++j)
        if (!(o.lam[j + 1] > o.lam[j])) return bad(err, "library ssp/" + lib.name + ": wavelengths must increase");
    long long off = 0;
    const long long ns = o.nspec, nt = o.nt, nz = o.nz;
    if (int rc = lib.check_array("stellar_mass", {zax, "log_age"}, {nz, nt}, off, err)) return rc;
    if (int rc = lib.read_real("stellar_mass", nt * nz, off, o.mass, err)) return rc;
    if (int rc = lib.check_array("spectra", {zax, "log_age", "wavelength"}, {nz, nt, ns}, off, err)) return rc;
    if (int rc = lib.read_real("spectra", ns * nt * nz, off, o.spec, err)) return rc;
    // log L_bol: the spectrum's trapezoid integral over frequency, floored at tiny
    std::vector<double> nu((size_t)ns);
    for (long long j = 0; j < ns; ++j) nu[(size_t)j] = o.lam[(size_t)j] > SAFE_FLOOR ? C_LIGHT / o.lam[(size_t)j] : 0.0;
    o.lbol.assign((size_t)(nt * nz), 0.0);
    for (long long k = 0; k < nt * nz; ++k)
        o.lbol[(size_t)k] = std::log10(std::max(trapz_abs(nu.data(), o.spec.data() + (size_t)(k * ns), (int)ns), SAFE_FLOOR));
    // nebular lines carried by the library (optional)
    o.nline = 0;
    o.line_lambda.clear();
    o.line_lum.clear();
    if (lib.has_array("line_luminosity")) {
        if (int rc = lib.axis_values("line_wavelength", o.line_lambda, err)) return rc;
        const long long nl = (long long)o.line_lambda.size();
        if (int rc = lib.check_array("line_luminosity", {zax, "log_age", "line_wavelength"}, {nz, nt, nl}, off, err)) return rc;
        if (int rc = lib.read_real("line_luminosity", nl * nt * nz, off, o.line_lum, err)) return rc;
        o.nline = (int)nl;
    }
    return 0;
}

int std_load_dust_emission(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                           std::vector<double> &qpah, std::vector<double> &umin, std::vector<double> &tab,
                           std::string &err) {
    DataLib lib;
    if (int rc = lib.open(root, "dust_emission", spec, err)) return rc;
    std::vector<double> wl;
    if (int rc = lib.axis_values("qpah", qpah, err)) return rc;
    if (int rc = lib.axis_values("umin", umin, err)) return rc;
    if (int rc = lib.axis_values("wavelength", wl, err)) return rc;
    const long long nq = (long long)qpah.size(), nu = (long long)umin.size(), nw = (long long)wl.size();
    if (nq < 2 || nu < 2 || nw < 2) return bad(err, "library dust_emission/" + lib.name + ": grid too small");
    long long off = 0;
    if (int rc = lib.check_array("spectra", {"qpah", "umin", "component", "wavelength"}, {nq, nu, 2, nw}, off, err)) return rc;
    std::vector<double> raw;
    if (int rc = lib.read_real("spectra", nq * nu * 2 * nw, off, raw, err)) return rc;
    const int ns = (int)lam.size();
    tab.assign((size_t)ns * nq * 2 * nu, 0.0);
    // the pixels from the one holding 1 um up (start_idx = max(find_interval(lambda, 1e4), 1))
    const int start = std::max(find_interval0(lam.data(), ns, 1.0e4), 0);
    for (long long q = 0; q < nq; ++q)
        for (long long col = 0; col < 2 * nu; ++col) {
            const double *y = raw.data() + (size_t)((q * 2 * nu + col) * nw);
            double *dst = tab.data() + (size_t)((col * nq + q) * ns);
            for (int p = start; p < ns; ++p) dst[p] = interp_linear(wl.data(), y, (int)nw, lam[(size_t)p]);
        }
    return 0;
}

int std_load_agn(const std::string &root, const std::vector<double> &lam, std::vector<double> &tau,
                 std::vector<double> &tab, std::string &err) {
    constexpr int NAGNDUST = 9;
    DataLib lib;
    if (int rc = lib.open(root, "agn_torus", "clumpy", err)) return rc;
    std::vector<double> wl;
    if (int rc = lib.axis_values("tau", tau, err)) return rc;
    if (int rc = lib.axis_values("wavelength", wl, err)) return rc;
    if ((int)tau.size() != NAGNDUST) return bad(err, "library agn_torus/clumpy: 9 optical depths are required");
    const long long nw = (long long)wl.size();
    if (nw < 2) return bad(err, "library agn_torus/clumpy: too few wavelengths");
    long long off = 0;
    if (int rc = lib.check_array("spectra", {"tau", "wavelength"}, {NAGNDUST, nw}, off, err)) return rc;
    std::vector<double> raw;
    if (int rc = lib.read_real("spectra", NAGNDUST * nw, off, raw, err)) return rc;
    const int ns = (int)lam.size();
    // pixels i1 .. i2 (1-based: max(find_interval(lambda, l_first), 1) .. max(find_interval(lambda, l_last), 1))
    const int i1 = std::max(find_interval0(lam.data(), ns, wl[0]), 0);
    const int i2 = std::max(find_interval0(lam.data(), ns, wl[(size_t)nw - 1]), 0);
    std::vector<double> lw((size_t)nw), ly((size_t)nw);
    for (long long i = 0; i < nw; ++i) lw[(size_t)i] = std::log10(wl[(size_t)i]);
    tab.assign((size_t)NAGNDUST * ns, 0.0);
    for (int t = 0; t < NAGNDUST; ++t) {
        for (long long i = 0; i < nw; ++i) ly[(size_t)i] = std::log10(raw[(size_t)(t * nw + i)] + SAFE_FLOOR);
        for (int p = i1; p <= i2 && p < ns; ++p)
            tab[(size_t)t * ns + p] = std::pow(10.0, interp_linear(lw.data(), ly.data(), (int)nw, std::log10(lam[(size_t)p]))) - SAFE_FLOOR;
    }
    return 0;
}

int std_load_attenuation(const std::string &root, const std::string &name, const std::vector<double> &lam,
                         std::vector<double> &tab, std::string &err) {
    const bool smc = name == "smc_bar";
    if (!smc && name != "dirty") return bad(err, "attenuation libraries: smc_bar or dirty", ST_BAD_ARG);
    DataLib lib;
    if (int rc = lib.open(root, "attenuation", name, err)) return rc;
    std::vector<double> wl;
    if (int rc = lib.axis_values("wavelength", wl, err)) return rc;
    const long long nw = (long long)wl.size();
    if (nw < 2) return bad(err, "library attenuation/" + name + ": too few wavelengths");
    if (!smc && nw != WG_NLAM) return bad(err, "library attenuation/dirty: 25 wavelengths are required");
    long long off = 0, ncurve = smc ? 1 : (long long)WG_NSTRUCT * WG_NTAU * WG_NMODEL;
    std::vector<double> raw;
    if (smc) {
        if (int rc = lib.check_array("extinction", {"wavelength"}, {nw}, off, err)) return rc;
        if (int rc = lib.read_real("extinction", nw, off, raw, err)) return rc;
    } else {
        if (int rc = lib.check_array("attenuation", {"structure", "tau_v", "model", "wavelength"},
                                     {WG_NSTRUCT, WG_NTAU, WG_NMODEL, nw}, off, err))
            return rc;
        if (int rc = lib.read_real("attenuation", ncurve * nw, off, raw, err)) return rc;
    }
    const size_t ns = lam.size();
    tab.assign((size_t)ncurve * ns, 0.0);
    for (long long k = 0; k < ncurve; ++k) {
        const double *y = raw.data() + (size_t)(k * nw);
        double *dst = tab.data() + (size_t)k * ns;
        for (size_t p = 0; p < ns; ++p) {
            const double l = lam[p];
            dst[p] = l > wl[(size_t)nw - 1] ? 0.0 : (l < wl[0] ? y[0] : interp_linear(wl.data(), y, (int)nw, l));
        }
    }
    return 0;
}

int std_load_nebular(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                     std::vector<double> &logz, std::vector<double> &lage, std::vector<double> &logu,
                     std::vector<double> &tab, std::string &err) {
    DataLib lib;
    if (int rc = lib.open(root, "nebular", spec, err)) return rc;
    std::vector<double> wl, age;
    if (int rc = lib.axis_values("logZ", logz, err)) return rc;
    if (int rc = lib.axis_values("age", age, err)) return rc;
    if (int rc = lib.axis_values("logU", logu, err)) return rc;
    if (int rc = lib.axis_values("wavelength", wl, err)) return rc;
    if ((int)logz.size() != NEB_NZ || (int)age.size() != NEB_NAGE || (int)logu.size() != NEB_NU)
        return bad(err, "library nebular/" + lib.name + ": the grid must be 11 logZ x 10 ages x 7 logU");
    const long long nw = (long long)wl.size();
    if (nw < 2) return bad(err, "library nebular/" + lib.name + ": too few wavelengths");
    for (double a : age)
        if (!(a > 0.0)) return bad(err, "library nebular/" + lib.name + ": ages must be positive");
    long long off = 0;
    if (int rc = lib.check_array("continuum", {"logZ", "age", "logU", "wavelength"}, {NEB_NZ, NEB_NAGE, NEB_NU, nw}, off,
                                 err))
        return rc;
    std::vector<double> raw;
    if (int rc = lib.read_real("continuum", (long long)NEB_NZ * NEB_NAGE * NEB_NU * nw, off, raw, err)) return rc;
    const int ns = (int)lam.size();
    tab.assign((size_t)ns * NEB_NZ * NEB_NAGE * NEB_NU, 0.0);
    std::vector<double> ly((size_t)nw);
    for (int z = 0; z < NEB_NZ; ++z)
        for (int a = 0; a < NEB_NAGE; ++a)
            for (int u = 0; u < NEB_NU; ++u) {
                const double *y = raw.data() + (size_t)(((z * NEB_NAGE + a) * NEB_NU + u) * nw);
                for (long long i = 0; i < nw; ++i) ly[(size_t)i] = std::log10(y[i] + 1.0e-95);
                double *dst = tab.data() + (size_t)ns * (z + NEB_NZ * (a + (size_t)NEB_NAGE * u));
                for (int p = 0; p < ns; ++p) dst[p] = interp_linear(wl.data(), ly.data(), (int)nw, lam[(size_t)p]);
            }
    lage.resize(age.size());
    for (size_t i = 0; i < age.size(); ++i) lage[i] = std::log10(age[i]);
    return 0;
}

int std_load_filters(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                     std::vector<double> &bands, std::vector<double> &pivot, std::vector<std::string> &names,
                     std::string &err) {
    DataLib lib;
    if (int rc = lib.open(root, "filters", spec, err)) return rc;
    long long nf = 0;
    if (int rc = lib.axis_len("filter", nf, err)) return rc;
    long long off = 0, lw = 0, lt = 0;
    if (int rc = lib.check_array("npoints", {"filter"}, {nf}, off, err)) return rc;
    std::vector<long long> npts;
    if (int rc = lib.read_int("npoints", nf, off, npts, err)) return rc;
    long long ntot = 0;
    bool neg = false;
    for (long long v : npts) { neg = neg || v < 0; ntot += v; }
    if (int rc = lib.array_len("wavelength", lw, err)) return rc;
    if (int rc = lib.array_len("transmission", lt, err)) return rc;
    if (neg || lw != ntot || lt != ntot)
        return bad(err, "filters/" + lib.name + ": wavelength and transmission must have sum(npoints) values");
    std::vector<double> all_l, all_t;
    if (int rc = lib.read_real("wavelength", ntot, 0, all_l, err)) return rc;
    if (int rc = lib.read_real("transmission", ntot, 0, all_t, err)) return rc;
    // per-filter metadata: names, detector, calibration {lambda_ref, exponent}
    std::vector<int> energy((size_t)nf, 0), has_cal((size_t)nf, 0);
    std::vector<double> cal_lref((size_t)nf, 0.0), cal_expo((size_t)nf, 0.0);
    names.assign((size_t)nf, std::string());
    if (const JVal *lab = lib.doc.get("axes")->get("filter")->get("labels"))
        for (size_t i = 0; i < lab->items.size() && i < (size_t)nf; ++i)
            if (lab->items[i].kind == JVal::STR) names[i] = lab->items[i].str;
    if (const JVal *fl = lib.meta("filters")) {
        if (fl->kind != JVal::ARR || (long long)fl->items.size() != nf)
            return bad(err, "filters/" + lib.name + ": metadata \"filters\" must have one entry per filter");
        for (long long i = 0; i < nf; ++i) {
            const JVal &e = fl->items[(size_t)i];
            if (const JVal *nm = e.get("name"))
                if (nm->kind == JVal::STR) names[(size_t)i] = nm->str;
            if (const JVal *dt = e.get("detector")) {
                if (dt->kind != JVal::STR || (dt->str != "photon" && dt->str != "energy"))
                    return bad(err, "filters/" + lib.name + ": filter " + std::to_string(i + 1) + ": detector must be \"photon\" or \"energy\"");
                energy[(size_t)i] = dt->str == "energy";
            }
            if (const JVal *cal = e.get("calibration")) {
                const JVal *lr = cal->get("lambda_ref"), *ex = cal->get("exponent");
                if (!lr || !ex || lr->kind != JVal::NUM || ex->kind != JVal::NUM || !(lr->num > 0.0))
                    return bad(err, "filters/" + lib.name + ": bad calibration of filter " + std::to_string(i + 1));
                has_cal[(size_t)i] = 1;
                cal_lref[(size_t)i] = lr->num;
                cal_expo[(size_t)i] = ex->num;
            }
        }
    }
    const int ng = (int)lam.size();
    bands.assign((size_t)nf * ng, 0.0);
    pivot.assign((size_t)nf, 0.0);
    std::vector<double> over((size_t)ng), lc, rc;
    long long first = 0;
    for (long long i = 0; i < nf; ++i) {
        // filter_clean (lenient): drop a point whose wavelength repeats the previous kept one, negative throughput
        // to zero
        lc.clear();
        rc.clear();
        for (long long k = 0; k < npts[(size_t)i]; ++k) {
            const double l = all_l[(size_t)(first + k)], r = all_t[(size_t)(first + k)];
            if (!lc.empty() && std::fabs(l - lc.back()) < SAFE_FLOOR) continue;
            lc.push_back(l);
            rc.push_back(std::max(r, 0.0));
        }
        first += npts[(size_t)i];
        const int nc = (int)lc.size();
        double *b = bands.data() + (size_t)i * ng;
        if (nc < 2) continue;                       // a dead filter: zero
        // resample_point: the legacy bounds, then the curve interpolated at each grid point in [si, ei]
        int si, ei;
        if (lc[0] <= lam[0]) si = 0;
        else si = std::max(find_interval0(lam.data(), ng, lc[0]) + 1, 1) - 1;
        if (lc[(size_t)nc - 1] >= lam[(size_t)ng - 1]) ei = ng - 1;
        else ei = std::min(find_interval0(lam.data(), ng, lc[(size_t)nc - 1]) + 1, ng) - 1;
        if (ei > si)
            for (int p = si; p <= ei; ++p) b[p] = interp_linear(lc.data(), rc.data(), nc, lam[(size_t)p]);
        if (energy[(size_t)i])
            for (int p = 0; p < ng; ++p) b[p] /= lam[(size_t)p];
        for (int p = 0; p < ng; ++p) b[p] = std::max(b[p], 0.0);
        for (int p = 0; p < ng; ++p) over[(size_t)p] = b[p] / (lam[(size_t)p] + SAFE_FLOOR);
        const double norm = trapz_abs(lam.data(), over.data(), ng);
        if (norm > SAFE_FLOOR) {
            for (int p = 0; p < ng; ++p) b[p] /= norm;
        } else {
            for (int p = 0; p < ng; ++p) b[p] = 0.0;
        }
        // filter_pivot: sqrt(int lambda T / int T / lambda)
        std::vector<double> lt2((size_t)ng), tl((size_t)ng);
        for (int p = 0; p < ng; ++p) { lt2[(size_t)p] = lam[(size_t)p] * b[p]; tl[(size_t)p] = b[p] / lam[(size_t)p]; }
        const double a = trapz_abs(lam.data(), lt2.data(), ng), d = trapz_abs(lam.data(), tl.data(), ng);
        pivot[(size_t)i] = (a != a || d != d || d <= SAFE_FLOOR) ? 0.0 : std::sqrt(a / d);
        // the calibration (apply_standard_filter_calibration, opensps_io.f90:1465-1500, filter_calibrate_band
        // opensps_filters.f90:505-518): divided by int (lambda / lambda_ref)^exponent T / lambda
        if (has_cal[(size_t)i]) {
            for (int p = 0; p < ng; ++p)
                over[(size_t)p] = std::pow(lam[(size_t)p] / cal_lref[(size_t)i], cal_expo[(size_t)i]) * b[p] / (lam[(size_t)p] + SAFE_FLOOR);
            const double dc = trapz_abs(lam.data(), over.data(), ng);
            if (dc > SAFE_FLOOR)
                for (int p = 0; p < ng; ++p) b[p] /= dc;
        }
    }
    return 0;
}

}  // namespace sps
