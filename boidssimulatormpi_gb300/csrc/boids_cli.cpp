// boids_cli.cpp -- Boost-free restatement of the reference's command line
// (src/args.cpp, src/main.cpp) over the C ABI of include/boids.h.
#include "boids_cli.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <vector>

#include "boids.h"

#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "frames are written in host byte order; the .ptcl format is little-endian"
#endif

namespace boidscli {

namespace {

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// [+-]? ( digits ('.' digits*)? | '.' digits ) ([eE] [+-]? digits)?  -- the
// forms std::num_get and lexical_cast read as a whole token.
bool is_decimal(const std::string &s)
{
    size_t i = 0, n = s.size();
    if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
    size_t d0 = i;
    while (i < n && std::isdigit((unsigned char)s[i])) ++i;
    size_t int_digits = i - d0, frac_digits = 0;
    if (i < n && s[i] == '.') {
        ++i;
        size_t f0 = i;
        while (i < n && std::isdigit((unsigned char)s[i])) ++i;
        frac_digits = i - f0;
    }
    if (int_digits + frac_digits == 0) return false;
    if (i < n && (s[i] == 'e' || s[i] == 'E')) {
        ++i;
        if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
        size_t e0 = i;
        while (i < n && std::isdigit((unsigned char)s[i])) ++i;
        if (i == e0) return false;
    }
    return i == n;
}

bool parse_magnitude(const std::string &s, size_t start, unsigned long long limit, unsigned long long &mag)
{
    if (start >= s.size()) return false;
    unsigned long long v = 0;
    for (size_t i = start; i < s.size(); ++i) {
        if (!std::isdigit((unsigned char)s[i])) return false;
        v = v * 10 + (unsigned)(s[i] - '0');
        if (v > limit) return false;
    }
    mag = v;
    return true;
}

}  // namespace

bool parse_unsigned(const std::string &s, unsigned &out)
{
    size_t i = 0;
    bool neg = false;
    if (!s.empty() && (s[0] == '+' || s[0] == '-')) {
        neg = s[0] == '-';
        i = 1;
    }
    unsigned long long m;
    if (!parse_magnitude(s, i, 0xffffffffull, m)) return false;
    out = neg ? (unsigned)(0u - (unsigned)m) : (unsigned)m;
    return true;
}

bool parse_int(const std::string &s, int &out)
{
    size_t i = 0;
    bool neg = false;
    if (!s.empty() && (s[0] == '+' || s[0] == '-')) {
        neg = s[0] == '-';
        i = 1;
    }
    unsigned long long m;
    if (!parse_magnitude(s, i, neg ? 2147483648ull : 2147483647ull, m)) return false;
    out = neg ? (int)(-(long long)m) : (int)m;
    return true;
}

bool parse_double(const std::string &s, double &out, bool allow_special)
{
    if (allow_special) {
        std::string t = s;
        bool neg = false;
        if (!t.empty() && (t[0] == '+' || t[0] == '-')) {
            neg = t[0] == '-';
            t = t.substr(1);
        }
        for (auto &c : t) c = (char)std::tolower((unsigned char)c);
        if (t == "inf" || t == "infinity") {
            out = neg ? -INFINITY : INFINITY;
            return true;
        }
        if (t == "nan") {
            out = neg ? -NAN : NAN;
            return true;
        }
    }
    if (!is_decimal(s)) return false;
    errno = 0;
    char *end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end != s.c_str() + s.size()) return false;
    if (errno == ERANGE && std::isinf(v)) return false;  // out of range: the stream sets failbit
    out = v;
    return true;
}

// ------------------------------------------------------------------ .ini

IniFile IniFile::parse(const std::string &text, const std::string &name)
{
    // property_tree read_ini: trimmed lines, ';' or '#' comments, "[section]"
    // headers, "key = value" pairs, no duplicate sections or keys.
    IniFile ini;
    std::istringstream in(text);
    std::string raw;
    unsigned line_no = 0;
    std::map<std::string, std::string> *cur = nullptr;
    auto err = [&](const std::string &what) {
        std::ostringstream o;
        o << (name.empty() ? "<unspecified file>" : name) << '(' << line_no << "): " << what;
        return std::runtime_error(o.str());
    };
    while (std::getline(in, raw)) {
        ++line_no;
        const std::string line = trim(raw);
        if (line.empty() || line[0] == ';' || line[0] == '#') continue;
        if (line[0] == '[') {
            const size_t end = line.find(']');
            if (end == std::string::npos) throw err("unmatched '['");
            const std::string sec = trim(line.substr(1, end - 1));
            if (ini.sections.count(sec) && !sec.empty()) throw err("duplicate section name");
            cur = &ini.sections[sec];
            continue;
        }
        std::map<std::string, std::string> &box = cur ? *cur : ini.sections[""];
        const size_t eq = line.find('=');
        if (eq == std::string::npos) throw err("'=' character not found in line");
        if (eq == 0) throw err("key expected");
        const std::string key = trim(line.substr(0, eq));
        const std::string val = trim(line.substr(eq + 1));
        if (box.count(key)) throw err("duplicate key name");
        box[key] = val;
    }
    return ini;
}

IniFile IniFile::read(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error((path.empty() ? "<unspecified file>" : path) + ": cannot open file");
    std::ostringstream s;
    s << f.rdbuf();
    return parse(s.str(), path);
}

const std::string *IniFile::find(const std::string &dotted) const
{
    const size_t dot = dotted.find('.');
    const std::string sec = dot == std::string::npos ? std::string() : dotted.substr(0, dot);
    const std::string key = dot == std::string::npos ? dotted : dotted.substr(dot + 1);
    auto s = sections.find(sec);
    if (s == sections.end()) return nullptr;
    auto k = s->second.find(key);
    return k == s->second.end() ? nullptr : &k->second;
}

void apply_ini(const IniFile &ini, Args &a)
{
    // get_optional<T>: a key whose value does not convert as a whole leaves
    // the parameter as it was (src/args.cpp:81-128).
    auto get_u = [&](const char *key, std::optional<unsigned> &dst) {
        unsigned v;
        if (const std::string *s = ini.find(key))
            if (parse_unsigned(*s, v)) dst = v;
    };
    auto get_i = [&](const char *key, std::optional<int> &dst) {
        int v;
        if (const std::string *s = ini.find(key))
            if (parse_int(*s, v)) dst = v;
    };
    auto get_d = [&](const char *key, std::optional<double> &dst) {
        double v;
        if (const std::string *s = ini.find(key))
            if (parse_double(*s, v, false)) dst = v;
    };
    get_u("Global.TIME_STEP", a.time_step);
    get_u("Global.POPULATION", a.population);
    get_d("Global.FIELD_SIZE", a.field_size);
    if (const std::string *s = ini.find("Global.INIT")) a.initialization = *s;
    get_i("Global.RANDOM_SEED", a.random_seed);
    get_d("Separation.SIGHT_DISTANCE", a.separation_sight_distance);
    get_d("Separation.SIGHT_ANGLE", a.separation_sight_angle);
    get_d("Separation.FORCE_COEFFICIENT", a.separation_force_coefficient);
    get_d("Alignment.SIGHT_DISTANCE", a.alignment_sight_distance);
    get_d("Alignment.SIGHT_ANGLE", a.alignment_sight_angle);
    get_d("Alignment.FORCE_COEFFICIENT", a.alignment_force_coefficient);
    get_d("Cohesion.SIGHT_DISTANCE", a.cohesion_sight_distance);
    get_d("Cohesion.SIGHT_ANGLE", a.cohesion_sight_angle);
    get_d("Cohesion.FORCE_COEFFICIENT", a.cohesion_force_coefficient);
    get_d("Velocity.MAX", a.velocity_max);
    get_d("Velocity.MIN", a.velocity_min);
}

// ------------------------------------------------------------------ command line

namespace {

enum OptId {
    O_HELP, O_SETTING, O_OUTPUT, O_VOUT, O_PAR, O_FORCE, O_INIT, O_N, O_T, O_F, O_VMIN, O_VMAX, O_SEED,
    O_INTERVAL, O_DEVICE, O_QUIET, O_PRINT, O_COUNT
};

struct Opt {
    OptId id;
    const char *name;
    char short_name;
    bool takes_value;
    const char *help;
};

// src/args.cpp:21-39, then the options of this build.
const Opt kOpts[] = {
    {O_HELP, "help", 'h', false, "help"},
    {O_SETTING, "setting", 's', true, "simulation setting file with .ini format."},
    {O_OUTPUT, "output", 'o', true, "output file."},
    {O_VOUT, "velocity-output", 0, true, "output file for velocity data."},
    {O_PAR, "parallel-output", 'p', false, "output data on several nodes on MPI (ignored: one GPU)."},
    {O_FORCE, "force-data-output", 0, false, "force vector output on data."},
    {O_INIT, "initialization", 'i', true,
     "initialization type or file name. if file name is given, simulation will start with last "
     "conditon of the file."},
    {O_N, "population", 'N', true, "Number of boids."},
    {O_T, "time-step", 'T', true, "Simulation time step."},
    {O_F, "field-size", 'F', true, "Size of simulation area."},
    {O_VMIN, "vmin", 0, true, "minimum velocity"},
    {O_VMAX, "vmax", 0, true, "maximum velocity"},
    {O_SEED, "random-seed", 0, true, "random seed"},
    {O_INTERVAL, "output-interval", 0, true, "write every k-th frame (default 1: every step)"},
    {O_DEVICE, "device", 0, true, "CUDA device ordinal (default 0)"},
    {O_QUIET, "quiet", 'q', false, "no per-step progress lines"},
    {O_PRINT, "print-config", 0, false, "print the resolved parameters and exit without running"},
};

std::string display(const Opt &o, bool as_short)
{
    if (as_short && o.short_name) return std::string("-") + o.short_name;
    return std::string("--") + o.name;
}

bool looks_like_option(const std::string &tok)
{
    if (tok.size() < 2 || tok[0] != '-') return false;
    double d;
    return !parse_double(tok, d, false);  // "-5" or "-0.1" is a value
}

}  // namespace

std::string usage(const char *prog)
{
    std::ostringstream o;
    o << "Usage: " << prog << " [options]\n\n";
    auto line = [&](const Opt &op) {
        std::string l = "  ";
        l += op.short_name ? std::string("-") + op.short_name + " [ --" + op.name + " ]" : std::string("--") + op.name;
        if (op.takes_value) l += " arg";
        if (l.size() < 34) l.resize(34, ' ');
        else l += ' ';
        o << l << op.help << '\n';
    };
    for (const Opt &op : kOpts)
        if (op.id <= O_FORCE) line(op);
    o << "\nsimulation parameters (have priority over setting file.):\n";
    for (const Opt &op : kOpts)
        if (op.id >= O_INIT && op.id <= O_SEED) line(op);
    o << "\nGB300 build options:\n";
    for (const Opt &op : kOpts)
        if (op.id > O_SEED) line(op);
    return o.str();
}

ParseResult parse_args(int argc, const char *const *argv, Args &a, std::string &err)
{
    std::optional<std::string> val[O_COUNT];
    bool seen[O_COUNT] = {};
    const Opt *shown[O_COUNT] = {};
    bool shown_short[O_COUNT] = {};
    std::vector<std::string> toks(argv + 1, argv + argc);

    auto occur = [&](const Opt &o, bool as_short, const std::optional<std::string> &v) -> bool {
        if (seen[o.id]) {
            err = "option '" + display(o, false) + "' cannot be specified more than once";
            return false;
        }
        seen[o.id] = true;
        shown[o.id] = &o;
        shown_short[o.id] = as_short;
        val[o.id] = v;
        return true;
    };

    for (size_t i = 0; i < toks.size(); ++i) {
        const std::string &t = toks[i];
        if (t == "--") {
            if (i + 1 < toks.size()) {
                err = "too many positional options have been specified on the command line";
                return PARSE_ERROR;
            }
            break;
        }
        if (t.size() > 2 && t[0] == '-' && t[1] == '-') {
            const size_t eq = t.find('=');
            const std::string name = t.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
            const Opt *hit = nullptr;
            std::vector<const Opt *> cands;
            for (const Opt &o : kOpts) {
                if (name == o.name) {
                    hit = &o;
                    break;
                }
                if (!name.empty() && std::strncmp(o.name, name.c_str(), name.size()) == 0) cands.push_back(&o);
            }
            if (!hit && cands.size() == 1) hit = cands[0];
            if (!hit && cands.size() > 1) {
                err = "option '--" + name + "' is ambiguous and matches ";
                for (size_t c = 0; c < cands.size(); ++c)
                    err += (c ? (c + 1 == cands.size() ? ", and '" : ", '") : "'") + display(*cands[c], false) + "'";
                return PARSE_ERROR;
            }
            if (!hit) {
                err = "unrecognised option '--" + name + "'";
                return PARSE_ERROR;
            }
            std::optional<std::string> v;
            if (hit->takes_value) {
                if (eq != std::string::npos) v = t.substr(eq + 1);
                else if (i + 1 < toks.size() && !looks_like_option(toks[i + 1])) v = toks[++i];
                else {
                    err = "the required argument for option '" + display(*hit, false) + "' is missing";
                    return PARSE_ERROR;
                }
            } else if (eq != std::string::npos) {
                err = "option '" + display(*hit, false) + "' does not take any arguments";
                return PARSE_ERROR;
            }
            if (!occur(*hit, false, v)) return PARSE_ERROR;
            continue;
        }
        if (t.size() >= 2 && t[0] == '-') {
            // -X, -Xvalue, -X value; switches may be stuck together (-hp)
            size_t pos = 1;
            while (pos < t.size()) {
                const char c = t[pos];
                const Opt *hit = nullptr;
                for (const Opt &o : kOpts)
                    if (o.short_name == c) hit = &o;
                if (!hit) {
                    err = std::string("unrecognised option '-") + c + "'";
                    return PARSE_ERROR;
                }
                std::optional<std::string> v;
                if (hit->takes_value) {
                    if (pos + 1 < t.size()) v = t.substr(pos + 1);
                    else if (i + 1 < toks.size() && !looks_like_option(toks[i + 1])) v = toks[++i];
                    else {
                        err = "the required argument for option '" + display(*hit, false) + "' is missing";
                        return PARSE_ERROR;
                    }
                    pos = t.size();
                } else {
                    ++pos;
                }
                if (!occur(*hit, true, v)) return PARSE_ERROR;
            }
            continue;
        }
        err = "too many positional options have been specified on the command line";
        return PARSE_ERROR;
    }

    // typed values (boost::lexical_cast)
    auto bad = [&](OptId id) {
        err = "the argument ('" + *val[id] + "') for option '" + display(*shown[id], false) + "' is invalid";
        return PARSE_ERROR;
    };
    unsigned u;
    int si;
    double d;
    std::optional<unsigned> cli_N, cli_T, cli_interval;
    std::optional<double> cli_F, cli_vmin, cli_vmax;
    std::optional<int> cli_seed, cli_device;
    if (seen[O_N]) { if (!parse_unsigned(*val[O_N], u)) return bad(O_N); cli_N = u; }
    if (seen[O_T]) { if (!parse_unsigned(*val[O_T], u)) return bad(O_T); cli_T = u; }
    if (seen[O_F]) { if (!parse_double(*val[O_F], d, true)) return bad(O_F); cli_F = d; }
    if (seen[O_VMIN]) { if (!parse_double(*val[O_VMIN], d, true)) return bad(O_VMIN); cli_vmin = d; }
    if (seen[O_VMAX]) { if (!parse_double(*val[O_VMAX], d, true)) return bad(O_VMAX); cli_vmax = d; }
    if (seen[O_SEED]) { if (!parse_int(*val[O_SEED], si)) return bad(O_SEED); cli_seed = si; }
    if (seen[O_INTERVAL]) {
        if (!parse_unsigned(*val[O_INTERVAL], u) || u == 0) return bad(O_INTERVAL);
        cli_interval = u;
    }
    if (seen[O_DEVICE]) { if (!parse_int(*val[O_DEVICE], si) || si < 0) return bad(O_DEVICE); cli_device = si; }
    (void)shown_short;

    if (seen[O_HELP]) return PARSE_HELP;  // src/args.cpp:52-55

    if (seen[O_SETTING]) a.setting_filename = *val[O_SETTING];
    if (seen[O_OUTPUT]) {
        a.output_filename = *val[O_OUTPUT];
        a.output_given = true;
    }
    if (seen[O_VOUT]) a.velocity_output_filename = *val[O_VOUT];
    a.is_parallel_output = false;  // src/args.cpp:62-67, non-MPI build
    a.is_force_data_output = seen[O_FORCE];
    a.quiet = seen[O_QUIET];
    a.print_config = seen[O_PRINT];
    if (seen[O_SETTING]) {
        try {
            apply_ini(IniFile::read(a.setting_filename), a);
        } catch (const std::exception &e) {
            err = e.what();
            return PARSE_ERROR;
        }
    }
    // command-line values over the .ini (src/args.cpp:130-153)
    if (seen[O_INIT]) {
        a.initialization = *val[O_INIT];
        a.initialization_given = true;
    }
    if (cli_F) a.field_size = cli_F;
    if (cli_N) a.population = cli_N;
    if (cli_T) a.time_step = cli_T;
    if (cli_vmin) a.velocity_min = cli_vmin;
    if (cli_vmax) a.velocity_max = cli_vmax;
    if (cli_seed) a.random_seed = cli_seed;
    if (cli_interval) a.output_interval = *cli_interval;
    if (cli_device) a.device = *cli_device;
    return PARSE_OK;
}

std::string format_config(const Args &a)
{
    std::ostringstream o;
    o.precision(17);
    auto put = [&](const char *k, const auto &v) {
        o << k << '=';
        if (v) o << *v;
        else o << "unset";
        o << '\n';
    };
    put("population", a.population);
    put("time_step", a.time_step);
    put("field_size", a.field_size);
    put("separation_sight_distance", a.separation_sight_distance);
    put("separation_sight_angle", a.separation_sight_angle);
    put("separation_force_coefficient", a.separation_force_coefficient);
    put("alignment_sight_distance", a.alignment_sight_distance);
    put("alignment_sight_angle", a.alignment_sight_angle);
    put("alignment_force_coefficient", a.alignment_force_coefficient);
    put("cohesion_sight_distance", a.cohesion_sight_distance);
    put("cohesion_sight_angle", a.cohesion_sight_angle);
    put("cohesion_force_coefficient", a.cohesion_force_coefficient);
    put("velocity_max", a.velocity_max);
    put("velocity_min", a.velocity_min);
    put("initialization", a.initialization);
    put("random_seed", a.random_seed);
    o << "output=" << a.output_filename << '\n'
      << "velocity_output=" << a.velocity_output_filename << '\n'
      << "force_data_output=" << (a.is_force_data_output ? 1 : 0) << '\n'
      << "output_interval=" << a.output_interval << '\n'
      << "device=" << a.device << '\n';
    return o.str();
}

// ------------------------------------------------------------------ .ptcl output

void encode_header(const PtclHeader &h, unsigned char out[50])
{
    // data_file_header_v02 (src/dtype.h:19-35), packed, little-endian
    auto u32 = [&](size_t off, uint32_t v) {
        for (int b = 0; b < 4; ++b) out[off + b] = (unsigned char)(v >> (8 * b));
    };
    auto f32 = [&](size_t off, float f) {
        uint32_t v;
        std::memcpy(&v, &f, 4);
        u32(off, v);
    };
    std::memcpy(out, "PTCL", 4);
    out[4] = 0;   // major_version
    out[5] = 2;   // minor_version
    u32(6, 50);   // header_length = sizeof(header)
    u32(10, h.n);
    u32(14, h.steps);
    u32(18, h.t0);
    u32(22, 30);  // FPS (src/main.cpp:17)
    f32(26, 0.0f);
    f32(30, h.field);
    f32(34, 0.0f);
    f32(38, h.field);
    f32(42, 0.0f);
    f32(46, h.field);
}

namespace {

// Frames leave the GPU through two page-locked buffers: while a writer
// thread waits for frame t's copy and writes it, the stream already runs
// update t and the copy of frame t+1 into the other buffer.
class FramePipe {
public:
    FramePipe(boids_sim *sim, size_t n, bool with_forces, std::FILE *fp, std::FILE *fv)
        : sim_(sim), pos_floats_(n * (with_forces ? 12 : 3)), vel_floats_(fv ? 3 * n : 0),
          with_forces_(with_forces), fp_(fp), fv_(fv)
    {
    }

    int start()
    {
        for (int s = 0; s < 2; ++s) {
            void *p = nullptr;
            if (boids_host_alloc(sizeof(float) * pos_floats_, &p)) return -1;
            hp_[s] = (float *)p;
            if (vel_floats_) {
                if (boids_host_alloc(sizeof(float) * vel_floats_, &p)) return -1;
                hv_[s] = (float *)p;
            }
        }
        th_ = std::thread([this] { writer(); });
        return 0;
    }

    // Queue the current state as the next frame.
    int submit()
    {
        const int slot = next_;
        next_ ^= 1;
        {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [&] { return !busy_[slot] || !error_.empty(); });
            if (!error_.empty()) return -1;
            busy_[slot] = true;
        }
        if (boids_frame_async(sim_, hp_[slot], vel_floats_ ? hv_[slot] : nullptr, with_forces_ ? 1 : 0, slot)) {
            std::lock_guard<std::mutex> lk(m_);
            busy_[slot] = false;
            error_ = boids_last_error();
            return -1;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            queue_.push_back(slot);
        }
        cv_.notify_all();
        return 0;
    }

    // Drain, stop the writer, free the buffers; returns the first error.
    std::string finish()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            done_ = true;
        }
        cv_.notify_all();
        if (th_.joinable()) th_.join();
        for (int s = 0; s < 2; ++s) {
            boids_host_free(hp_[s]);
            boids_host_free(hv_[s]);
            hp_[s] = hv_[s] = nullptr;
        }
        return error_;
    }

    ~FramePipe() { finish(); }

private:
    void writer()
    {
        for (;;) {
            int slot;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return !queue_.empty() || done_; });
                if (queue_.empty()) return;
                slot = queue_.front();
                queue_.pop_front();
            }
            std::string e;
            if (boids_frame_wait(sim_, slot)) e = boids_last_error();
            // each frame is flushed, as src/main.cpp:281-284 does
            if (e.empty() && (std::fwrite(hp_[slot], sizeof(float), pos_floats_, fp_) != pos_floats_ ||
                              std::fflush(fp_) != 0))
                e = "write failed on the output file";
            if (e.empty() && fv_ &&
                (std::fwrite(hv_[slot], sizeof(float), vel_floats_, fv_) != vel_floats_ || std::fflush(fv_) != 0))
                e = "write failed on the velocity output file";
            {
                std::lock_guard<std::mutex> lk(m_);
                busy_[slot] = false;
                if (!e.empty() && error_.empty()) error_ = e;
            }
            cv_.notify_all();
        }
    }

    boids_sim *sim_;
    size_t pos_floats_, vel_floats_;
    bool with_forces_;
    std::FILE *fp_, *fv_;
    float *hp_[2] = {nullptr, nullptr}, *hv_[2] = {nullptr, nullptr};
    int next_ = 0;
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<int> queue_;
    bool busy_[2] = {false, false};
    bool done_ = false;
    std::string error_;
    std::thread th_;
};

struct SimGuard {
    boids_sim *s = nullptr;
    ~SimGuard()
    {
        if (s) boids_destroy(s);
    }
};

struct FileGuard {
    std::FILE *f = nullptr;
    ~FileGuard()
    {
        if (f) std::fclose(f);
    }
};

}  // namespace

int run(const Args &a, int engine, const char *prog)
{
    const char *missing = nullptr;
    if (!a.population) missing = "POPULATION / -N";
    else if (!a.time_step) missing = "TIME_STEP / -T";
    else if (!a.field_size) missing = "FIELD_SIZE / -F";
    else if (!a.separation_sight_distance || !a.separation_sight_angle || !a.separation_force_coefficient)
        missing = "[Separation] SIGHT_DISTANCE, SIGHT_ANGLE, FORCE_COEFFICIENT";
    else if (!a.alignment_sight_distance || !a.alignment_sight_angle || !a.alignment_force_coefficient)
        missing = "[Alignment] SIGHT_DISTANCE, SIGHT_ANGLE, FORCE_COEFFICIENT";
    else if (!a.cohesion_sight_distance || !a.cohesion_sight_angle || !a.cohesion_force_coefficient)
        missing = "[Cohesion] SIGHT_DISTANCE, SIGHT_ANGLE, FORCE_COEFFICIENT";
    else if (!a.velocity_max || !a.velocity_min) missing = "[Velocity] MIN, MAX / --vmin, --vmax";
    const std::string init = a.initialization ? *a.initialization : std::string();
    const bool drawn = init == "test" || init == "random_uniform";
    if (!missing && drawn && engine == BOIDS_ENGINE_GRID && !a.random_seed) missing = "RANDOM_SEED / --random-seed";
    if (missing) {
        // the reference reads an indeterminate value here
        std::cerr << prog << ": parameter not set: " << missing << std::endl;
        return -1;
    }
    if (a.initialization_given && !a.output_given) {
        // src/args.cpp:32 binds -i to the output file name too, so the
        // reference would truncate the initialization file it just read
        std::cerr << prog << ": --initialization without --output would overwrite the initialization file; "
                  << "give -o" << std::endl;
        return -1;
    }

    boids_params p{};
    p.number_of_agents = *a.population;
    p.field_size = *a.field_size;
    p.separation_sight_distance = *a.separation_sight_distance;
    p.separation_sight_angle = *a.separation_sight_angle;
    p.separation_force_coefficient = *a.separation_force_coefficient;
    p.alignment_sight_distance = *a.alignment_sight_distance;
    p.alignment_sight_angle = *a.alignment_sight_angle;
    p.alignment_force_coefficient = *a.alignment_force_coefficient;
    p.cohesion_sight_distance = *a.cohesion_sight_distance;
    p.cohesion_sight_angle = *a.cohesion_sight_angle;
    p.cohesion_force_coefficient = *a.cohesion_force_coefficient;
    p.velocity_max = *a.velocity_max;
    p.velocity_min = *a.velocity_min;
    p.engine = engine;
    p.device = a.device;
    p.flags = a.is_force_data_output ? BOIDS_FLAG_RECORD_FORCES : 0u;

    SimGuard sim;
    if (boids_create(&p, &sim.s)) {
        std::cerr << boids_last_error() << std::endl;
        return -1;
    }
    if (engine == BOIDS_ENGINE_GRID) {  // src/boid_simulation_grid.cpp:91-92
        boids_grid_info gi{};
        boids_get_grid_info(sim.s, &gi);
        std::cout << "# Grid List Optimization enabled" << std::endl << "  grid num:" << gi.ref_grid_num << std::endl;
    }
    if (boids_init(sim.s, init.c_str(), a.random_seed ? *a.random_seed : 0)) {
        std::cerr << boids_last_error() << std::endl;
        return -1;
    }
    // src/main.cpp:96-121
    std::cout << "N: " << p.number_of_agents << std::endl
              << "field size: " << p.field_size << "," << p.field_size << "," << p.field_size << std::endl
              << "#Separation" << std::endl
              << "force: " << p.separation_force_coefficient << std::endl
              << "area distance: " << p.separation_sight_distance << std::endl
              << "area angle: " << p.separation_sight_angle << std::endl
              << "#Alignment" << std::endl
              << "force: " << p.alignment_force_coefficient << std::endl
              << "area distance: " << p.alignment_sight_distance << std::endl
              << "area angle: " << p.alignment_sight_angle << std::endl
              << "#Cohesion" << std::endl
              << "force: " << p.cohesion_force_coefficient << std::endl
              << "area distance: " << p.cohesion_sight_distance << std::endl
              << "area angle: " << p.cohesion_sight_angle << std::endl
              << "#Velocity" << std::endl
              << "min: " << p.velocity_min << std::endl
              << "max: " << p.velocity_max << std::endl
              << "#CUDA: " << boids_version() << ", device " << a.device << std::endl;

    // src/main.cpp:157-175
    FileGuard fout, vout;
    fout.f = std::fopen(a.output_filename.c_str(), "wb");
    if (!fout.f) {
        std::cerr << "Couldn't open: " << a.output_filename << std::endl;
        return -1;
    }
    const bool with_v = !a.velocity_output_filename.empty();
    if (with_v) {
        vout.f = std::fopen(a.velocity_output_filename.c_str(), "wb");
        if (!vout.f) {
            std::cerr << "Couldn't open: " << a.velocity_output_filename << std::endl;
            return -1;
        }
    }
    const unsigned T = *a.time_step, k = a.output_interval;
    const unsigned frames = T / k + (T % k ? 1u : 0u);  // k == 1: T frames, as the reference writes
    unsigned char hdr[50];
    encode_header(PtclHeader{p.number_of_agents, frames, 0u, (float)p.field_size}, hdr);
    if (std::fwrite(hdr, 1, 50, fout.f) != 50 || (with_v && std::fwrite(hdr, 1, 50, vout.f) != 50)) {
        std::cerr << prog << ": write failed" << std::endl;
        return -1;
    }

    std::cout << "simulation start." << std::endl;
    FramePipe pipe(sim.s, p.number_of_agents, a.is_force_data_output, fout.f, with_v ? vout.f : nullptr);
    if (pipe.start()) {
        std::cerr << boids_last_error() << std::endl;
        return -1;
    }
    // src/main.cpp:187-292: the frame of step t is the state before update t
    for (unsigned t = 0; t < T; ++t) {
        if (t % k == 0 && pipe.submit()) break;
        if (!a.quiet) std::cout << "  " << t << "/" << T << std::endl;
        if (boids_step(sim.s, 1)) {
            std::cerr << boids_last_error() << std::endl;
            pipe.finish();
            return -1;
        }
    }
    const std::string err = pipe.finish();
    if (!err.empty()) {
        std::cerr << prog << ": " << err << std::endl;
        return -1;
    }
    if (boids_synchronize(sim.s)) {
        std::cerr << boids_last_error() << std::endl;
        return -1;
    }
    std::cout << "simulation finished." << std::endl;
    return 0;
}

}  // namespace boidscli
