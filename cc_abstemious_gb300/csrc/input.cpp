// Input layer: the JSON UserInput (input_data.rs:9-108, serde_json with
// externally tagged enums), the VTK legacy ASCII reader in the reference
// dialect (mesh_data.rs:96-175) and the frequency lists (preprocess.rs:155-167,
// tools.rs:1-24).  Host C++; no JSON library is available, so a small
// recursive-descent parser is included.
#include <atomic>
#include <charconv>
#include <cstdio>
#include <type_traits>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

#include "common.cuh"

namespace bem {
namespace {

struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0;
    bool is_integer = false;  // literal without fraction or exponent
    bool negative = false;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;
    const JValue* get(const std::string& k) const {
        for (auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

class JParser {
  public:
    explicit JParser(const std::string& s) : s_(s) {}
    JValue parse() {
        JValue v = value(0);
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    const std::string& s_;
    size_t i_ = 0;
    [[noreturn]] void fail(const std::string& m) {
        throw Error(BEM_ERR_BAD_INPUT, "JSON parse error at offset " + std::to_string(i_) + ": " + m);
    }
    void ws() {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
    }
    JValue value(int depth) {
        if (depth > 64) fail("nesting too deep");
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        char c = s_[i_];
        JValue v;
        if (c == '{') {
            v.kind = JValue::Object;
            ++i_;
            ws();
            if (i_ < s_.size() && s_[i_] == '}') { ++i_; return v; }
            for (;;) {
                ws();
                if (i_ >= s_.size() || s_[i_] != '"') fail("expected key");
                std::string k = string();
                ws();
                if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':'");
                ++i_;
                JValue e = value(depth + 1);
                v.obj.emplace_back(k, std::move(e));
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
                if (i_ < s_.size() && s_[i_] == '}') { ++i_; break; }
                fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.kind = JValue::Array;
            ++i_;
            ws();
            if (i_ < s_.size() && s_[i_] == ']') { ++i_; return v; }
            for (;;) {
                v.arr.push_back(value(depth + 1));
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
                if (i_ < s_.size() && s_[i_] == ']') { ++i_; break; }
                fail("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.kind = JValue::String;
            v.str = string();
        } else if (s_.compare(i_, 4, "true") == 0) {
            v.kind = JValue::Bool; v.b = true; i_ += 4;
        } else if (s_.compare(i_, 5, "false") == 0) {
            v.kind = JValue::Bool; v.b = false; i_ += 5;
        } else if (s_.compare(i_, 4, "null") == 0) {
            v.kind = JValue::Null; i_ += 4;
        } else if (c == '-' || std::isdigit((unsigned char)c)) {
            size_t st = i_;
            if (s_[i_] == '-') { v.negative = true; ++i_; }
            if (i_ >= s_.size() || !std::isdigit((unsigned char)s_[i_])) fail("bad number");
            while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
            bool integer = true;
            if (i_ < s_.size() && s_[i_] == '.') {
                integer = false;
                ++i_;
                if (i_ >= s_.size() || !std::isdigit((unsigned char)s_[i_])) fail("bad number");
                while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
            }
            if (i_ < s_.size() && (s_[i_] == 'e' || s_[i_] == 'E')) {
                integer = false;
                ++i_;
                if (i_ < s_.size() && (s_[i_] == '+' || s_[i_] == '-')) ++i_;
                if (i_ >= s_.size() || !std::isdigit((unsigned char)s_[i_])) fail("bad number");
                while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
            }
            v.kind = JValue::Number;
            v.is_integer = integer;
            v.num = std::strtod(s_.c_str() + st, nullptr);
        } else {
            fail("unexpected character");
        }
        return v;
    }
    std::string string() {
        ++i_;  // opening quote
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c == '\\') {
                if (i_ >= s_.size()) fail("bad escape");
                char e = s_[i_++];
                switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    if (i_ + 4 > s_.size()) fail("bad \\u escape");
                    unsigned cp = (unsigned)std::strtoul(s_.substr(i_, 4).c_str(), nullptr, 16);
                    i_ += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: fail("bad escape");
                }
            } else {
                out += c;
            }
        }
        if (i_ >= s_.size()) fail("unterminated string");
        ++i_;
        return out;
    }
};

// serde_json typing rules: f64 accepts any number; usize only non-negative
// integer literals.
double as_f64(const JValue* v, const char* what) {
    require(v != nullptr, std::string("missing field `") + what + "`");
    require(v->kind == JValue::Number, std::string("invalid type for `") + what + "`, expected f64");
    return v->num;
}
int64_t as_usize(const JValue* v, const char* what) {
    require(v != nullptr, std::string("missing field `") + what + "`");
    require(v->kind == JValue::Number && v->is_integer && !v->negative,
            std::string("invalid type for `") + what + "`, expected usize");
    return (int64_t)v->num;
}
const JValue& field(const JValue& o, const char* name) {
    require(o.kind == JValue::Object, std::string("expected struct containing `") + name + "`");
    const JValue* v = o.get(name);
    require(v != nullptr, std::string("missing field `") + name + "`");
    return *v;
}
void fixed_array(const JValue& a, double* out, size_t n, const char* what) {
    require(a.kind == JValue::Array && a.arr.size() == n,
            std::string("invalid length for `") + what + "`, expected an array of length " + std::to_string(n));
    for (size_t i = 0; i < n; ++i) out[i] = as_f64(&a.arr[i], what);
}

// Externally tagged enum: unit variants are strings, struct variants are
// single-key objects.
std::pair<std::string, const JValue*> tagged(const JValue& v, const char* what) {
    if (v.kind == JValue::String) return {v.str, nullptr};
    require(v.kind == JValue::Object && v.obj.size() == 1,
            std::string("invalid type for enum `") + what + "`");
    return {v.obj[0].first, &v.obj[0].second};
}

int unit_variant(const JValue& v, const char* what, std::initializer_list<const char*> names) {
    auto t = tagged(v, what);
    int idx = 0;
    for (const char* n : names) {
        if (t.first == n) return idx;
        ++idx;
    }
    throw Error(BEM_ERR_BAD_INPUT, std::string("unknown variant `") + t.first + "` for `" + what + "`");
}

}  // namespace

UserInput parse_user_input(const std::string& text) {
    JValue root = JParser(text).parse();
    require(root.kind == JValue::Object, "input must be a JSON object");
    UserInput u;
    const JValue& mf = field(root, "mesh_file");
    require(mf.kind == JValue::String, "invalid type for `mesh_file`, expected a string");
    u.mesh_file = mf.str;
    u.body_index = as_usize(&field(root, "body_index"), "body_index");
    {   // FrequencyInput (input_data.rs:9-14)
        auto t = tagged(field(root, "frequency"), "frequency");
        require(t.second != nullptr, "frequency must be a struct variant");
        if (t.first == "List") {
            u.freq_kind = 0;
            const JValue& vals = field(*t.second, "values");
            require(vals.kind == JValue::Array, "invalid type for `values`");
            for (auto& x : vals.arr) u.freq_values.push_back(as_f64(&x, "values"));
        } else if (t.first == "LinearSpaced" || t.first == "LogSpaced") {
            u.freq_kind = t.first == "LinearSpaced" ? 1 : 2;
            u.freq_start = as_f64(t.second->get("start"), "start");
            u.freq_end = as_f64(t.second->get("end"), "end");
            u.freq_number = as_usize(t.second->get("number"), "number");
        } else {
            throw Error(BEM_ERR_BAD_INPUT, "unknown variant `" + t.first + "` for `frequency`");
        }
    }
    u.sound_speed = as_f64(root.get("sound_speed"), "sound_speed");
    u.mass_density = as_f64(root.get("mass_density"), "mass_density");
    u.problem_type = unit_variant(field(root, "problem_type"), "problem_type", {"Interior", "Exterior"});
    u.method_type = unit_variant(field(root, "method_type"), "method_type", {"Classical", "BurtonMiller"});
    {   // Solver (input_data.rs:29-34) + additive optional H-matrix keys
        auto t = tagged(field(root, "solver"), "solver");
        require(t.second != nullptr && t.second->kind == JValue::Object, "solver must be a struct variant");
        if (t.first == "Direct") {
            u.solver = 0;
        } else if (t.first == "Iterative" || t.first == "Hierarchical") {
            u.solver = t.first == "Iterative" ? 1 : 2;
            u.tolerance = as_f64(t.second->get("tolerance"), "tolerance");
            u.max_iterations = as_usize(t.second->get("max_iterations"), "max_iterations");
            if (const JValue* l = t.second->get("leaf_size")) u.hm_leaf = as_usize(l, "leaf_size");
            if (const JValue* e = t.second->get("eta")) u.hm_eta = as_f64(e, "eta");
            if (const JValue* a = t.second->get("aca_tolerance")) u.hm_aca_tol = as_f64(a, "aca_tolerance");
        } else {
            throw Error(BEM_ERR_BAD_INPUT, "unknown variant `" + t.first + "` for `solver`");
        }
    }
    {   // IncidentWaveInput (input_data.rs:36-46)
        auto wave = [](const JValue& v, const char* key) {
            auto t = tagged(v, key);
            require(t.second != nullptr, std::string(key) + " must be a struct variant");
            UserInput::Wave w{};
            if (t.first == "PlaneWave") {
                w.type = 0;
                fixed_array(field(*t.second, "direction"), w.vec, 3, "direction");
            } else if (t.first == "SphericalWave") {
                w.type = 1;
                fixed_array(field(*t.second, "origin"), w.vec, 3, "origin");
            } else {
                throw Error(BEM_ERR_BAD_INPUT, "unknown variant `" + t.first + "` for `" + key + "`");
            }
            fixed_array(field(*t.second, "amplitude"), w.amp, 2, "amplitude");
            return w;
        };
        u.waves.push_back(wave(field(root, "incident_wave"), "incident_wave"));
        // extension: further right-hand sides solved with the same operators
        // (unknown to the reference, whose serde ignores the key)
        if (const JValue* extra = root.get("additional_incident_waves")) {
            require(extra->kind == JValue::Array, "additional_incident_waves must be an array");
            for (const JValue& v : extra->arr) u.waves.push_back(wave(v, "additional_incident_waves"));
        }
        const UserInput::Wave& w0 = u.waves[0];
        u.incident_type = w0.type;
        for (int k = 0; k < 3; ++k) u.incident_vec[k] = w0.vec[k];
        u.incident_amp[0] = w0.amp[0];
        u.incident_amp[1] = w0.amp[1];
    }
    {   // SurfaceBoundaryCondition (input_data.rs:48-59)
        const JValue& bc = field(root, "surface_bc");
        u.bc_type = unit_variant(field(bc, "bc_type"), "bc_type", {"Pressure", "NormalVelocity", "Impedance"});
        fixed_array(field(bc, "value"), u.bc_value, 2, "value");
    }
    {   // Output (input_data.rs:61-78)
        const JValue& o = field(root, "output");
        u.output_total = unit_variant(field(o, "o_type"), "o_type", {"Scattered", "Total"});
        u.output_pressure = unit_variant(field(o, "field"), "field", {"VelocityPotential", "Pressure"});
        const JValue& f = field(o, "file");
        require(f.kind == JValue::String, "invalid type for `file`");
        u.output_file = f.str;
        const JValue& fps = field(o, "field_points");
        require(fps.kind == JValue::Array, "invalid type for `field_points`");
        for (auto& p : fps.arr) {
            double xyz[3];
            fixed_array(p, xyz, 3, "field_points");
            u.field_points.insert(u.field_points.end(), xyz, xyz + 3);
        }
    }
    return u;
}

// mesh_data.rs:96-175: line-oriented reader; POINTS rows carry 3 coordinates,
// CELLS rows carry the body id then the node ids, CELL_TYPES one type per row.
namespace {
// Line-oriented cursor over a file held in memory.
struct Lines {
    const char* p;
    const char* end;
    bool next(const char*& b, const char*& e) {
        if (p >= end) return false;
        b = p;
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        e = nl ? nl : end;
        p = nl ? nl + 1 : end;
        return true;
    }
};

// Host threads for parsing large mesh blocks, created on first use and kept
// for the life of the process (the pool is never destroyed; its threads wait
// on a condition variable).  A process forked after creation has no workers
// and parses on the calling thread.
class RowPool {
  public:
    static RowPool& get() {
        static RowPool* p = new RowPool();
        return *p;
    }
    int size() const { return getpid() == owner_ ? (int)threads_.size() + 1 : 1; }
    // f(t) for t in [0, n), n <= size(), t = 0 on the calling thread; returns
    // when all are done
    void run(int n, const std::function<void(int)>& f) {
        if (n <= 1) {
            if (n == 1) f(0);
            return;
        }
        std::lock_guard<std::mutex> serial(serial_);
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &f;
            n_ = n;
            next_ = 1;
            pending_ = n - 1;
            ++gen_;
        }
        cv_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

  private:
    RowPool() : owner_(getpid()) {
        const unsigned hw = std::thread::hardware_concurrency();
        const unsigned nw = std::min(7u, hw > 1 ? hw - 1 : 0u);
        for (unsigned i = 0; i < nw; ++i) threads_.emplace_back([this] { loop(); });
    }
    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
            cv_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            while (next_ < n_) {
                const int t = next_++;
                const std::function<void(int)>* f = job_;
                lk.unlock();
                (*f)(t);
                lk.lock();
                if (--pending_ == 0) done_.notify_one();
            }
        }
    }
    pid_t owner_;
    std::vector<std::thread> threads_;
    std::mutex m_, serial_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* job_ = nullptr;
    int n_ = 0, next_ = 0, pending_ = 0;
    uint64_t gen_ = 0;
};

// The next n rows of a block: their [begin, end) spans, the cursor moved past
// them.  False if the text ends first.
bool take_rows(Lines& L, int64_t n, std::vector<const char*>& lb, std::vector<const char*>& le) {
    lb.resize((size_t)n);
    le.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i)
        if (!L.next(lb[(size_t)i], le[(size_t)i])) return false;
    return true;
}

// Splits rows [0, n) into contiguous chunks over the pool (one chunk per
// ~1024 rows); row(chunk, i) parses row i and returns false on a bad row.
// Returns the first bad row, or -1.  The results do not depend on the split.
template <class F>
int64_t parallel_rows(int64_t n, int nt, F row) {
    std::vector<int64_t> bad((size_t)nt, -1);
    RowPool::get().run(nt, [&](int t) {
        const int64_t i0 = n * t / nt, i1 = n * (t + 1) / nt;
        for (int64_t i = i0; i < i1; ++i)
            if (!row(t, i)) {
                bad[(size_t)t] = i;
                return;
            }
    });
    for (int64_t b : bad)
        if (b >= 0) return b;
    return -1;
}

int chunks_for(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(RowPool::get().size(), n / 1024));
}

inline const char* skip_ws(const char* s, const char* e) {
    while (s < e && (*s == ' ' || *s == '\t' || *s == '\r')) ++s;
    return s;
}

// One number; false at the end of the line or on a non-number.  from_chars
// is correctly rounded like strtod; a form it rejects (a leading '+') goes
// through strtod on a bounded copy.
template <class T>
inline bool parse_num(const char*& s, const char* e, T& v) {
    s = skip_ws(s, e);
    if (s >= e) return false;
    auto r = std::from_chars(s, e, v);
    if (r.ec == std::errc() && r.ptr != s) {
        s = r.ptr;
        return true;
    }
    char buf[64];
    size_t n = 0;
    while (s + n < e && n < sizeof(buf) - 1 && s[n] != ' ' && s[n] != '\t' && s[n] != '\r') ++n;
    std::memcpy(buf, s, n);
    buf[n] = 0;
    char* q = nullptr;
    if constexpr (std::is_floating_point<T>::value) v = (T)std::strtod(buf, &q);
    else v = (T)std::strtoll(buf, &q, 10);
    if (q == buf) return false;
    s += (q - buf);
    return true;
}

inline std::string first_word(const char* b, const char* e) {
    b = skip_ws(b, e);
    const char* w = b;
    while (w < e && *w != ' ' && *w != '\t' && *w != '\r') ++w;
    return std::string(b, w);
}
}  // namespace

void host_parallel_for(int64_t n, const std::function<void(int64_t)>& f) {
    if (n <= 0) return;
    const int nt = (int)std::min<int64_t>(RowPool::get().size(), n);
    std::atomic<int64_t> next{0};
    std::mutex m;
    std::exception_ptr err;
    RowPool::get().run(nt, [&](int) {
        for (int64_t i; (i = next.fetch_add(1)) < n;) {
            try {
                f(i);
            } catch (...) {
                std::lock_guard<std::mutex> lk(m);
                if (!err) err = std::current_exception();
            }
        }
    });
    if (err) std::rethrow_exception(err);
}

Mesh read_vtk(const std::string& path) {
    std::string text;
    {
        FILE* fp = std::fopen(path.c_str(), "rb");
        require(fp != nullptr, "Mesh file not found at specified path: " + path);
        std::fseek(fp, 0, SEEK_END);
        const long sz = std::ftell(fp);
        std::fseek(fp, 0, SEEK_SET);
        text.resize(sz > 0 ? (size_t)sz : 0);
        const size_t got = sz > 0 ? std::fread(&text[0], 1, (size_t)sz, fp) : 0;
        std::fclose(fp);
        require(got == text.size(), "VTK: cannot read " + path);
    }
    // error messages are built only on failure (they would cost an allocation
    // per number otherwise)
    auto fail = [](const char* what, const char* lb, const char* le) {
        throw Error(BEM_ERR_BAD_INPUT, std::string(what) + std::string(lb, le));
    };
    Lines L{text.data(), text.data() + text.size()};
    Mesh m;
    const char *b, *e;
    std::vector<const char*> lb, le;  // rows of the current block
    auto count_after = [&](const char* lb, const char* le) -> int64_t {
        const char* s = skip_ws(lb, le);
        while (s < le && *s != ' ' && *s != '\t') ++s;  // the keyword
        long long n = -1;
        if (!parse_num(s, le, n) || n < 0) fail("VTK: bad block header: ", lb, le);
        return (int64_t)n;
    };
    while (L.next(b, e)) {
        const std::string w = first_word(b, e);
        if (w == "POINTS") {
            const int64_t n = count_after(b, e);
            m.nodes.assign((size_t)(3 * n), 0.0);
            if (!take_rows(L, n, lb, le)) fail("VTK: unexpected end of POINTS", b, b);
            const int64_t bad = parallel_rows(n, chunks_for(n), [&](int, int64_t i) {
                const char* s = lb[(size_t)i];
                for (int c = 0; c < 3; ++c)
                    if (!parse_num(s, le[(size_t)i], m.nodes[(size_t)(3 * i + c)])) return false;
                return true;
            });
            if (bad >= 0) fail("VTK: bad point row: ", lb[(size_t)bad], le[(size_t)bad]);
        } else if (w == "CELLS") {
            const int64_t n = count_after(b, e);
            m.body.assign((size_t)n, 0);
            m.etype.assign((size_t)n, 0);
            m.conn_off.assign((size_t)n + 1, 0);
            m.conn.clear();
            if (!take_rows(L, n, lb, le)) fail("VTK: unexpected end of CELLS", b, b);
            // node ids per chunk, then concatenated in row order
            const int nt = chunks_for(n);
            struct alignas(64) Part {  // one cache line per chunk's vector header
                std::vector<int64_t> v;
            };
            std::vector<Part> part((size_t)nt);
            for (auto& q : part) q.v.reserve((size_t)(4 * n / nt + 16));
            std::vector<int64_t> cnt((size_t)n, 0);
            const int64_t bad = parallel_rows(n, nt, [&](int t, int64_t i) {
                const char* s = lb[(size_t)i];
                long long bv;
                if (!parse_num(s, le[(size_t)i], bv)) return false;
                m.body[(size_t)i] = bv;
                long long v;
                std::vector<int64_t>& out = part[(size_t)t].v;
                const size_t before = out.size();
                while (parse_num(s, le[(size_t)i], v)) out.push_back(v);
                cnt[(size_t)i] = (int64_t)(out.size() - before);
                return true;
            });
            if (bad >= 0) fail("VTK: bad cell row: ", lb[(size_t)bad], le[(size_t)bad]);
            for (int64_t i = 0; i < n; ++i) m.conn_off[(size_t)i + 1] = m.conn_off[(size_t)i] + cnt[(size_t)i];
            m.conn.reserve((size_t)m.conn_off[(size_t)n]);
            for (auto& q : part) m.conn.insert(m.conn.end(), q.v.begin(), q.v.end());
        } else if (w == "CELL_TYPES") {
            const int64_t n = count_after(b, e);
            require(n <= m.nelem(), "VTK: CELL_TYPES longer than CELLS");
            for (int64_t i = 0; i < n; ++i) {
                const char *lb, *le;
                if (!L.next(lb, le)) fail("VTK: unexpected end of CELL_TYPES", b, b);
                const char* s = lb;
                long v = 0;
                parse_num(s, le, v);
                m.etype[(size_t)i] = (int32_t)v;
            }
        }
    }
    // bodies in order of first appearance (mesh_data.rs:163-171)
    for (int64_t e = 0; e < m.nelem(); ++e) {
        int64_t b = m.body[(size_t)e];
        require(b >= 1, "VTK: body ids start at 1");
        if (b > m.nbodies) {
            require(b == m.nbodies + 1, "VTK: body ids must appear in increasing order without gaps");
            m.nbodies++;
        }
    }
    return m;
}

// tools.rs:1-24 linspace / logspace with exact endpoints.
static std::vector<double> linspace(double start, double end, int64_t n) {
    std::vector<double> x((size_t)n, start);
    double dx = (end - start) / (double)(n - 1);
    for (int64_t i = 1; i < n - 1; ++i) x[(size_t)i] = start + dx * (double)i;
    x[(size_t)n - 1] = end;
    return x;
}

// Tuning table (tuning.json, written by cc_abstemious_gb300/tune.py):
// {"entries": [{"kernel": K, "n": N, "nsys": S, "params": {name: int, ...}}, ...]}
std::vector<TuneEntry> parse_tuning(const std::string& text) {
    JValue root = JParser(text).parse();
    require(root.kind == JValue::Object, "tuning table: expected an object");
    const JValue* ents = root.get("entries");
    require(ents && ents->kind == JValue::Array, "tuning table: missing `entries`");
    std::vector<TuneEntry> out;
    for (const JValue& e : ents->arr) {
        require(e.kind == JValue::Object, "tuning table: entries must be objects");
        TuneEntry t;
        const JValue* k = e.get("kernel");
        const JValue* n = e.get("n");
        const JValue* ns = e.get("nsys");
        const JValue* ps = e.get("params");
        require(k && k->kind == JValue::String && n && n->kind == JValue::Number && ns &&
                    ns->kind == JValue::Number && ps && ps->kind == JValue::Object,
                "tuning table: an entry needs kernel, n, nsys and params");
        t.kernel = k->str;
        t.n = (int64_t)n->num;
        t.nsys = (int64_t)ns->num;
        for (auto& kv : ps->obj) {
            require(kv.second.kind == JValue::Number, "tuning table: parameters are integers");
            t.params.emplace_back(kv.first, (int)kv.second.num);
        }
        out.push_back(std::move(t));
    }
    return out;
}

int TuningTable::get(const char* kernel, const char* param, int64_t n, int64_t nsys, int dflt) const {
    // the entry of this kernel that sets the parameter, nearest in log(n),
    // then log(nsys)
    const TuneEntry* best = nullptr;
    double bd = 0;
    for (const TuneEntry& e : entries) {
        if (e.kernel != kernel) continue;
        bool has = false;
        for (auto& kv : e.params) has = has || kv.first == param;
        if (!has) continue;
        const double d = std::fabs(std::log((double)std::max<int64_t>(n, 1) / (double)std::max<int64_t>(e.n, 1))) +
                         0.25 * std::fabs(std::log((double)std::max<int64_t>(nsys, 1) /
                                                   (double)std::max<int64_t>(e.nsys, 1)));
        if (!best || d < bd) {
            best = &e;
            bd = d;
        }
    }
    if (!best) return dflt;
    for (auto& kv : best->params)
        if (kv.first == param) return kv.second;
    return dflt;
}

std::vector<double> frequency_list(const UserInput& in) {
    if (in.freq_kind == 0) return in.freq_values;
    require(in.freq_number >= 1, "frequency: number must be at least 1");
    if (in.freq_kind == 1) return linspace(in.freq_start, in.freq_end, in.freq_number);
    std::vector<double> xl = linspace(std::log10(in.freq_start), std::log10(in.freq_end), in.freq_number);
    std::vector<double> x((size_t)in.freq_number, in.freq_start);
    x[(size_t)in.freq_number - 1] = in.freq_end;
    for (int64_t i = 1; i < in.freq_number - 1; ++i) x[(size_t)i] = std::pow(10.0, xl[(size_t)i]);
    return x;
}

}  // namespace bem
