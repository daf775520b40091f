// Output path: the CSV writers of postprocess.rs:15-67.  Numbers are written
// the way Rust's `f64::to_string()` (Display) writes them: the shortest
// decimal digits that round-trip, laid out in positional notation (no
// exponent; zeros pad large and small magnitudes), no decimal point for
// integral values ("1", "-0", "0.0000001", "100000000000000000000000" for
// 1e23), "NaN" / "inf" / "-inf".  The digits come from std::to_chars in
// scientific format without a precision (shortest round-trip, closest on
// ties); the positional layout is written here.  Records are comma-separated
// and end with "\n" (the csv 1.3.1 crate's Writer defaults: no field here
// needs quoting).
#include <charconv>
#include <cmath>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "common.cuh"

namespace bem {

std::string rust_f64(double v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    char buf[64];
    const std::to_chars_result r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    require(r.ec == std::errc(), "formatting a number failed", BEM_ERR_CUDA);
    // d[.ddd]e(+|-)xx -> sign, the digits, the decimal exponent of the first
    const std::string sci(buf, r.ptr);
    std::string out = sci[0] == '-' ? "-" : "";
    const size_t b = out.size(), e = sci.find('e');
    std::string digits;
    for (size_t i = b; i < e; ++i)
        if (sci[i] != '.') digits += sci[i];
    const int point = std::stoi(sci.substr(e + 1)) + 1;  // digits before the decimal point
    const int nd = (int)digits.size();
    if (point <= 0) out += "0." + std::string((size_t)(-point), '0') + digits;
    else if (point >= nd) out += digits + std::string((size_t)(point - nd), '0');
    else out += digits.substr(0, (size_t)point) + "." + digits.substr((size_t)point);
    return out;
}

namespace {

struct CsvFile {
    FILE* f = nullptr;
    explicit CsvFile(const std::string& path) {
        f = std::fopen(path.c_str(), "wb");
        require(f != nullptr, "cannot create output file " + path);
    }
    void record(const std::vector<std::string>& fields) {
        std::string line;
        for (size_t i = 0; i < fields.size(); ++i) {
            if (i) line += ',';
            line += fields[i];
        }
        line += '\n';
        require(std::fwrite(line.data(), 1, line.size(), f) == line.size(), "writing the output file failed");
    }
    ~CsvFile() {
        if (f) std::fclose(f);
    }
};

std::string output_path(const Problem& p, const char* path) {
    std::string out = path ? std::string(path) : p.in.output_file;
    require(!out.empty(), "no output file: the input's output.file is empty and no path was given");
    return out;
}

// postprocess.rs:24-27: "pre" for pressure, "vpo" for velocity potential
std::string field_name(const Problem& p) { return p.in.output_pressure ? "pre" : "vpo"; }

template <class F>
bem_status guarded(bem_ctx* ctx, F&& f) {
    try {
        f();
        return BEM_OK;
    } catch (const Error& e) {
        if (ctx) ctx->c.last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        if (ctx) ctx->c.last_error = e.what();
        return BEM_ERR_BAD_INPUT;
    }
}

}  // namespace
}  // namespace bem

using namespace bem;

extern "C" {

BEM_API bem_status bem_write_results_at_frequency(bem_ctx* ctx, const bem_problem* pp, const char* path,
                                                  const bem_cplx* scattered, const bem_cplx* incident) {
    if (!pp || !scattered || !incident) return BEM_ERR_BAD_INPUT;
    return guarded(ctx, [&] {
        const Problem& p = pp->p;
        CsvFile w(output_path(p, path));
        const std::string on = field_name(p);
        w.record({"index", "x", "y", "z", on + "_re", on + "_im", "inc_re", "inc_im"});
        const int64_t nfp = (int64_t)p.in.field_points.size() / 3;
        for (int64_t i = 0; i < nfp; ++i) {
            const double* x = p.in.field_points.data() + 3 * i;
            w.record({std::to_string(i), rust_f64(x[0]), rust_f64(x[1]), rust_f64(x[2]), rust_f64(scattered[i].re),
                      rust_f64(scattered[i].im), rust_f64(incident[i].re), rust_f64(incident[i].im)});
        }
    });
}

BEM_API bem_status bem_write_results_at_point(bem_ctx* ctx, const bem_problem* pp, const char* path, int64_t index,
                                              const bem_cplx* scattered, const bem_cplx* incident) {
    if (!pp || !scattered || !incident) return BEM_ERR_BAD_INPUT;
    return guarded(ctx, [&] {
        const Problem& p = pp->p;
        const int64_t nfp = (int64_t)p.in.field_points.size() / 3;
        require(index >= 0 && index < nfp, "field point index out of range");
        CsvFile w(output_path(p, path));
        const std::string on = field_name(p);
        w.record({"freq", on + "_re", on + "_im", "inc_re", "inc_im"});
        for (size_t f = 0; f < p.freqs.size(); ++f) {
            const size_t o = f * (size_t)nfp + (size_t)index;
            w.record({rust_f64(p.freqs[f]), rust_f64(scattered[o].re), rust_f64(scattered[o].im),
                      rust_f64(incident[o].re), rust_f64(incident[o].im)});
        }
    });
}

BEM_API int64_t bem_format_f64(double v, char* buf, int64_t len) {
    std::string s;
    try {
        s = rust_f64(v);
    } catch (...) {
        return -1;
    }
    if (buf && len > 0) {
        const size_t k = std::min<size_t>(s.size(), (size_t)(len - 1));
        std::memcpy(buf, s.data(), k);
        buf[k] = '\0';
    }
    return (int64_t)s.size();
}

}  // extern "C"
