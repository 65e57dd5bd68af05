// config.cpp -- the .sph-config reader (sim/config-parser.go).
//
// Two passes as in the reference: a tokenizer (sim/config-parser.go:486-679)
// producing [[Title]], [Subtitle], integer, float, vec2 and word tokens with
// line/column positions, then a validating pass (sim/config-parser.go:186-432)
// mapping (title, subtitle, name) onto SphConfig fields. Messages keep the
// reference's "file:line:col: ConfigParseError|ConfigMakeError: ..." format
// and wording (including its spelling) so tools matching on them keep working.
// Where the reference panics (unreadable file, a number or word at the very
// end of the file, an unparsable "-" literal, a character no rule accepts)
// this reader returns a ConfigParseError instead.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sphgpu.h"

namespace {

enum TokType { T_TITLE = 0, T_SUBTITLE, T_INTEGER, T_FLOAT, T_VEC2, T_WORD };

// names printed by the reference's generated String() (sim/tokentype_string.go:
// the word type post-dates the generated table, so it prints as TokenType(5))
const char *tok_type_name(int t) {
    static const char *names[] = {"title", "subtitle", "integer", "float", "vec2", "TokenType(5)"};
    return (t >= 0 && t <= 5) ? names[t] : "TokenType(?)";
}

struct Token {
    int type = 0;
    std::string str, name;
    int64_t ival = 0;
    double fval = 0;
    double v2[2] = {0, 0};
    int line = 0, row = 0;
};

struct ConfigError {
    std::string msg;
};

bool is_letter(uint32_t c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'); }
bool is_digit(uint32_t c) { return c >= '0' && c <= '9'; }
// unicode.IsSpace for the Latin-1 range plus the common Unicode spaces
bool is_space(uint32_t c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r' || c == 0x85 || c == 0xA0 ||
           c == 0x1680 || (c >= 0x2000 && c <= 0x200a) || c == 0x2028 || c == 0x2029 || c == 0x202f ||
           c == 0x205f || c == 0x3000;
}
bool is_hspace(uint32_t c) { return is_space(c) && c != '\n'; }

std::vector<uint32_t> decode_utf8(const std::string &s) {
    std::vector<uint32_t> out;
    size_t i = 0;
    while (i < s.size()) {
        unsigned char c = (unsigned char)s[i];
        uint32_t cp;
        int len;
        if (c < 0x80) { cp = c; len = 1; }
        else if ((c >> 5) == 6) { cp = c & 0x1f; len = 2; }
        else if ((c >> 4) == 14) { cp = c & 0x0f; len = 3; }
        else if ((c >> 3) == 30) { cp = c & 0x07; len = 4; }
        else { out.push_back(0xfffd); i++; continue; }
        if (i + len > s.size()) { out.push_back(0xfffd); break; }
        bool ok = true;
        for (int j = 1; j < len; j++) {
            unsigned char d = (unsigned char)s[i + j];
            if ((d >> 6) != 2) { ok = false; break; }
            cp = (cp << 6) | (d & 0x3f);
        }
        if (!ok) { out.push_back(0xfffd); i++; continue; }
        out.push_back(cp);
        i += len;
    }
    return out;
}

std::string encode_utf8(uint32_t c) {
    std::string s;
    if (c < 0x80) s += (char)c;
    else if (c < 0x800) { s += (char)(0xc0 | (c >> 6)); s += (char)(0x80 | (c & 0x3f)); }
    else if (c < 0x10000) {
        s += (char)(0xe0 | (c >> 12)); s += (char)(0x80 | ((c >> 6) & 0x3f)); s += (char)(0x80 | (c & 0x3f));
    } else {
        s += (char)(0xf0 | (c >> 18)); s += (char)(0x80 | ((c >> 12) & 0x3f));
        s += (char)(0x80 | ((c >> 6) & 0x3f)); s += (char)(0x80 | (c & 0x3f));
    }
    return s;
}

std::string str_of(const std::vector<uint32_t> &v, size_t a, size_t b) {
    std::string s;
    for (size_t i = a; i < b; i++) s += encode_utf8(v[i]);
    return s;
}

// A cursor over the file's runes with the reference's line bookkeeping:
// `line` counts newlines consumed, `bol` is the cursor at the line start.
struct Tokenizer {
    std::string fname;
    std::vector<uint32_t> text;
    size_t pos = 0;
    int line = 0;
    size_t bol = 0;

    bool eof() const { return pos >= text.size(); }
    uint32_t cur() const { return text[pos]; }
    void chop(size_t n) {
        for (size_t i = 0; i < n && pos < text.size(); i++) {
            uint32_t r = text[pos++];
            if (r == '\n') { line++; bol = pos; }
        }
    }
    ConfigError parse_error(const std::string &msg) const {
        std::ostringstream o;
        o << fname << ":" << line + 1 << ":" << (pos - bol + 1) << ": ConfigParseError: " << msg << "\n";
        return ConfigError{o.str()};
    }
    template <typename F>
    size_t chop_until_nofail(F pred) {
        size_t a = pos;
        while (!eof() && !pred(cur())) chop(1);
        return a;
    }
    template <typename F>
    size_t chop_until(F pred, const std::string &expect) {
        size_t a = chop_until_nofail(pred);
        if (eof()) throw parse_error("Expected " + expect + ", but got to the end of the file");
        return a;
    }
    void trim_all() { while (!eof() && is_space(cur())) chop(1); }
    void trim_h() { while (!eof() && is_hspace(cur())) chop(1); }
    void expect(uint32_t r) {
        if (eof()) throw parse_error("Expected `" + encode_utf8(r) + "`, but got to the end of the file");
        if (cur() != r) throw parse_error("Expected `" + encode_utf8(r) + "`, but we got this: `" + encode_utf8(cur()) + "`");
    }
};

std::vector<Token> tokenize(const std::string &fname) {
    std::ifstream f(fname, std::ios::binary);
    if (!f) {
        std::ostringstream o;
        o << fname << ":1:1: ConfigParseError: cannot read the file\n";
        throw ConfigError{o.str()};
    }
    std::stringstream ss;
    ss << f.rdbuf();
    Tokenizer t;
    t.fname = fname;
    t.text = decode_utf8(ss.str());
    std::vector<Token> toks;
    auto not_letter = [](uint32_t c) { return !is_letter(c); };
    auto not_digit = [](uint32_t c) { return !is_digit(c); };
    for (;;) {
        t.trim_all();
        if (t.eof()) break;
        if (t.cur() == '/') {
            t.chop(1);
            t.expect('/');
            t.chop(1);
            t.chop_until_nofail([](uint32_t c) { return c == '\n'; });
            if (t.eof()) break;
        } else if (t.cur() == '[') {
            t.chop(1);
            if (t.eof()) throw t.parse_error("Expected a Title starting with `[[` or a Subtitle starting with `[` and then at least one letter");
            if (is_letter(t.cur())) {
                int row = (int)(t.pos - t.bol + 1);
                size_t a = t.chop_until(not_letter, "a letter or `]`");
                std::string content = str_of(t.text, a, t.pos);
                t.expect(']');
                t.chop(1);
                Token k;
                k.type = T_SUBTITLE;
                k.str = content;
                k.line = t.line + 1;
                k.row = row;
                toks.push_back(k);
            } else if (t.cur() == '[') {
                t.chop(1);
                int row = (int)(t.pos - t.bol + 1);
                size_t a = t.chop_until(not_letter, "a letter or `]]`");
                std::string content = str_of(t.text, a, t.pos);
                if (content.empty()) throw t.parse_error("Expected a letter after `[[` but got `" + encode_utf8(t.cur()) + "`");
                t.expect(']');
                t.chop(1);
                t.expect(']');
                t.chop(1);
                Token k;
                k.type = T_TITLE;
                k.str = content;
                k.line = t.line + 1;
                k.row = row;
                toks.push_back(k);
            } else {
                throw t.parse_error("Expected a Title starting with `[[` or a Subtitle starting with `[` and then at least one letter");
            }
        } else if (is_letter(t.cur())) {
            size_t a = t.chop_until(not_letter, "a letter as start of a parmeter name");
            std::string name = str_of(t.text, a, t.pos);
            int row = (int)(t.pos - t.bol + 1);
            t.trim_h();
            if (t.eof()) throw t.parse_error("`" + name + "` Excpected a Number/Vec2 or Word");
            if (is_digit(t.cur()) || t.cur() == '-') {
                std::vector<std::string> parts;
                bool any_float = false;
                for (;;) {
                    t.trim_h();
                    bool neg = false;
                    if (!t.eof() && t.cur() == '-') { neg = true; t.chop(1); }
                    if (!parts.empty() && (t.eof() || t.cur() == '\n')) break;
                    size_t l0 = t.chop_until_nofail(not_digit);
                    std::string left = (neg ? "-" : "") + str_of(t.text, l0, t.pos);
                    if (!t.eof() && t.cur() == '.') {
                        t.chop(1);
                        size_t r0 = t.chop_until(not_digit, "that there is no digit here");
                        parts.push_back(left + "." + str_of(t.text, r0, t.pos));
                        any_float = true;
                    } else if (t.eof() || is_space(t.cur())) {
                        parts.push_back(left);
                    } else {
                        throw t.parse_error("In number literal expected a `.` or a digit");
                    }
                    if (parts.size() > 2) throw t.parse_error("Cannot parse a Vector with more than 2 dimensions");
                    if (t.eof()) break;
                }
                Token k;
                k.name = name;
                k.line = t.line + 1;
                k.row = row;
                auto parse_f = [&](const std::string &s) {
                    char *end = nullptr;
                    double v = strtod(s.c_str(), &end);
                    if (s.empty() || s == "-" || s == "." || s == "-." || *end) throw t.parse_error("invalid number literal `" + s + "`");
                    return v;
                };
                if (parts.size() == 1) {
                    if (any_float) {
                        k.type = T_FLOAT;
                        k.fval = parse_f(parts[0]);
                    } else {
                        char *end = nullptr;
                        const std::string &s = parts[0];
                        long long v = strtoll(s.c_str(), &end, 10);
                        if (s.empty() || s == "-" || *end) throw t.parse_error("invalid integer literal `" + s + "`");
                        k.type = T_INTEGER;
                        k.ival = v;
                    }
                } else {
                    k.type = T_VEC2;
                    k.v2[0] = parse_f(parts[0]);
                    k.v2[1] = parse_f(parts[1]);
                }
                toks.push_back(k);
            } else if (is_letter(t.cur())) {
                size_t w0 = t.chop_until_nofail(not_letter);
                std::string word = str_of(t.text, w0, t.pos);
                if (word.empty() || (!t.eof() && !is_space(t.cur())))
                    throw t.parse_error("`" + word + "` Excpected only Letters and a whitespace at the end to form a Word");
                Token k;
                k.type = T_WORD;
                k.name = name;
                k.str = word;
                k.line = t.line + 1;
                k.row = row;
                toks.push_back(k);
            } else {
                throw t.parse_error("`" + name + "` Excpected a Number/Vec2 or Word");
            }
        } else {
            throw t.parse_error("unimplemented - starts with: `" + encode_utf8(t.cur()) + "`");
        }
    }
    return toks;
}

struct Maker {
    std::string fname;
    ConfigError err(const Token &t, const std::string &msg) const {
        std::ostringstream o;
        o << fname << ":" << t.line << ":" << t.row << ": ConfigMakeError: " << msg << "\n";
        return ConfigError{o.str()};
    }
    int64_t get_int(const Token &t) const {
        if (t.type != T_INTEGER) throw err(t, "expected an integer but got something else");
        return t.ival;
    }
    double get_float(const Token &t) const {
        if (t.type != T_INTEGER && t.type != T_FLOAT) throw err(t, "expected an integer or float but got something else");
        return t.type == T_INTEGER ? (double)t.ival : t.fval;
    }
    void get_vec2(const Token &t, double out[2]) const {
        if (t.type != T_VEC2) throw err(t, "expected an integer but got something else");
        out[0] = t.v2[0];
        out[1] = t.v2[1];
    }
};

const char *const kTitles[] = {"Simulation", "Start", "Boundaries", "Sources"};
const char *const kSubs[4][2] = {{"Config", "Viewport"}, {"UniformRect", nullptr}, {"Periodic", "Reflection"}, {"Point", nullptr}};

int title_index(const std::string &s) {
    for (int i = 0; i < 4; i++) if (s == kTitles[i]) return i;
    return -1;
}
bool valid_sub(int ti, const std::string &s) {
    for (int j = 0; j < 2; j++) if (kSubs[ti][j] && s == kSubs[ti][j]) return true;
    return false;
}
std::string subs_list(int ti) {
    std::string s = "[";
    for (int j = 0; j < 2; j++) {
        if (!kSubs[ti][j]) continue;
        if (j) s += " ";
        s += kSubs[ti][j];
    }
    return s + "]";
}

void update_from_tokens(sph_config *cfg, std::vector<Token> toks, const std::string &fname) {
    Maker M{fname};
    size_t i = 0;
    while (i < toks.size()) {
        Token tok = toks[i++];
        if (tok.type != T_TITLE) throw M.err(tok, std::string("Expected a [[Title]] but got `") + tok_type_name(tok.type) + "`");
        const std::string title = tok.str;
        int ti = title_index(title);
        if (ti < 0) throw M.err(tok, "`" + title + "` is not a valid title");
        if (i >= toks.size()) break;
        tok = toks[i++];
        if (tok.type != T_SUBTITLE) throw M.err(tok, std::string("Expected a [Subtitle] but got `") + tok_type_name(tok.type) + "`");
        std::string sub = tok.str;
        if (!valid_sub(ti, sub))
            throw M.err(tok, "`" + sub + "` is not a valid subtitle under title: `" + title + "`. It's valid subtitles are: " + subs_list(ti));
        if (i >= toks.size()) break;
        while (i < toks.size()) {
            if (toks[i].type == T_TITLE) break;
            tok = toks[i++];
            if (tok.type == T_SUBTITLE) {
                sub = tok.str;
                if (!valid_sub(ti, sub))
                    throw M.err(tok, "`" + sub + "` is not a valid subtitle under title: `" + title + "`. It's valid subtitles incude: " + subs_list(ti));
                continue;
            }
            const std::string &nm = tok.name;
            sph_params &p = cfg->params;
            if (title == "Simulation" && sub == "Config") {
                if (nm == "NSteps") cfg->nsteps = (int32_t)M.get_int(tok);
                else if (nm == "Gamma") p.gamma = M.get_float(tok);
                else if (nm == "ParticleMass") p.mass = M.get_float(tok);
                else if (nm == "DeltaTHalf") p.dth = M.get_float(tok);
                else if (nm == "Acceleration") M.get_vec2(tok, p.accel);
                else if (nm == "Kernel") {
                    const std::string k = tok.type == T_WORD ? tok.str : std::string();
                    if (k == "Monahan") p.kernel = SPH_KERNEL_MONAHAN;
                    else if (k == "Wendtland") p.kernel = SPH_KERNEL_WENDLAND;
                    else throw M.err(tok, "Kernel `" + k + "` is not implemented");
                }
                // keys this library adds for the parameters the reference hard-codes
                else if (nm == "NeighbourCount") p.k = (int32_t)M.get_int(tok);
                else if (nm == "ViscosityAlpha") p.alpha = M.get_float(tok);
                else if (nm == "ViscosityBeta") p.beta = M.get_float(tok);
                else if (nm == "ViscosityEtaSq") p.etasq = M.get_float(tok);
                else if (nm == "GridLevel") p.grid_level = (int32_t)M.get_int(tok);
                else if (nm == "Precision") {
                    const std::string w = tok.type == T_WORD ? tok.str : std::string();
                    if (w == "Exact") p.precision = SPH_PREC_FP64;
                    else if (w == "Fast") p.precision = SPH_PREC_FP64_FAST;
                    else if (w == "Mixed") p.precision = SPH_PREC_MIXED;
                    else throw M.err(tok, "Precision `" + w + "` is not implemented");
                } else throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
            } else if (title == "Simulation" && sub == "Viewport") {
                // the reference assigns these without checking the token type
                double v[2] = {0, 0};
                if (tok.type == T_VEC2) { v[0] = tok.v2[0]; v[1] = tok.v2[1]; }
                if (nm == "UpperLeft") { cfg->viewport[0] = v[0]; cfg->viewport[1] = v[1]; }
                else if (nm == "LowerRight") { cfg->viewport[2] = v[0]; cfg->viewport[3] = v[1]; }
                else throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
            } else if (title == "Start" && sub == "UniformRect") {
                if (nm != "NParticles" && nm != "UpperLeft" && nm != "LowerRight")
                    throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
                if (toks.size() - i < 2)
                    throw M.err(tok, "Expected 3 Params following [`" + sub + "`] but got something else or nothing.\n\tOne of each paramas `NParticles, UpperLeft, LowerRight` must be defined");
                sph_rect_spawner sp;
                memset(&sp, 0, sizeof sp);
                // the reference records the FIRST parameter's name three times
                // (sim/config-parser.go:330), so only a repeat of it is caught
                std::vector<std::string> got(3);
                const std::string first = nm;
                for (int r = 0; r < 3; r++) {
                    for (const auto &g : got)
                        if (g == tok.name) throw M.err(tok, "The parameter name `" + tok.name + "` in [`" + sub + "`] is already set!");
                    if (tok.type != T_INTEGER && tok.type != T_VEC2)
                        throw M.err(tok, "Expected either an integer or vec2 parameter definition in [`" + sub + "`], but got `" + tok_type_name(tok.type) + "`");
                    if (tok.name == "NParticles") sp.n = M.get_int(tok);
                    else if (tok.name == "UpperLeft") M.get_vec2(tok, sp.upper_left);
                    else if (tok.name == "LowerRight") M.get_vec2(tok, sp.lower_right);
                    else throw M.err(tok, "The parameter name `" + tok.name + "` in [`" + sub + "`] is not valid. Needs to be one of `NParticles, UpperLeft, LowerRight`");
                    got.push_back(first);
                    if (r == 2) break;
                    tok = toks[i++];
                }
                if (i < toks.size() && toks[i].type != T_TITLE && toks[i].type != T_SUBTITLE)
                    throw M.err(tok, "The 4th parameter name `" + tok.name + "` in [`" + sub + "`] is too much. need to have `NParticles, UpperLeft and LowerRight`");
                if (cfg->nstart >= SPH_CONFIG_MAX_SPAWNERS) throw M.err(tok, "too many [UniformRect] spawners");
                cfg->start[cfg->nstart++] = sp;
            } else if (title == "Boundaries" && sub == "Periodic") {
                double v[2];
                if (nm == "Vertical") { M.get_vec2(tok, v); cfg->params.vert[0] = v[0]; cfg->params.vert[1] = v[1]; }
                else if (nm == "Horizontal") { M.get_vec2(tok, v); cfg->params.hor[0] = v[0]; cfg->params.hor[1] = v[1]; }
                else throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
            } else if (title == "Boundaries" && sub == "Reflection") {
                if (nm == "Left") cfg->params.refl[0] = M.get_float(tok);
                else if (nm == "Right") cfg->params.refl[1] = M.get_float(tok);
                else if (nm == "Up") cfg->params.refl[2] = M.get_float(tok);
                else if (nm == "Down") cfg->params.refl[3] = M.get_float(tok);
                else throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
            } else if (title == "Sources" && sub == "Point") {
                if (nm != "Pos" && nm != "Rate")
                    throw M.err(tok, "`" + nm + "` is not a valid parameter in `[[" + title + "]]` - `[" + sub + "]`");
                sph_point_source ps;
                memset(&ps, 0, sizeof ps);
                if (nm == "Pos") {
                    M.get_vec2(tok, ps.origin);
                    if (i >= toks.size()) throw M.err(tok, "Expected `rate` but got nothing");
                    tok = toks[i++];
                    ps.rate = M.get_float(tok);
                } else {
                    ps.rate = M.get_float(tok);
                    if (i >= toks.size()) throw M.err(tok, "Expected `pos` but got nothing");
                    tok = toks[i++];
                    M.get_vec2(tok, ps.origin);
                }
                if (cfg->nsources >= SPH_CONFIG_MAX_SPAWNERS) throw M.err(tok, "too many [Point] sources");
                cfg->sources[cfg->nsources++] = ps;
            }
        }
    }
}

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (double)(next() >> 11) * 0x1.0p-53; }
};

}  // namespace

extern "C" {

sph_params sph_default_params(void);

void sph_config_default(sph_config *out) {
    if (!out) return;
    memset(out, 0, sizeof *out);
    out->params = sph_default_params();
    out->nsteps = 10000;
    out->viewport[0] = 0;
    out->viewport[1] = 0;
    out->viewport[2] = 1;
    out->viewport[3] = 1;
}

int sph_config_load(const char *path, sph_config *out, char *err, int32_t errlen) {
    if (!out || !path) return SPH_ERR_ARG;
    sph_config_default(out);
    try {
        std::vector<Token> toks = tokenize(path);
        update_from_tokens(out, toks, path);
    } catch (const ConfigError &e) {
        sph_config_default(out);
        if (err && errlen > 0) {
            strncpy(err, e.msg.c_str(), (size_t)errlen - 1);
            err[errlen - 1] = 0;
        }
        return SPH_ERR_CONFIG;
    }
    if (err && errlen > 0) err[0] = 0;
    return SPH_OK;
}

int64_t sph_config_start_count(const sph_config *cfg) {
    if (!cfg) return -1;
    int64_t n = 0;
    for (int i = 0; i < cfg->nstart; i++) n += cfg->start[i].n > 0 ? cfg->start[i].n : 0;
    return n;
}

int sph_config_spawn(const sph_config *cfg, double *x, double *y, double *vx, double *vy, double *u, int64_t *z) {
    if (!cfg || !x || !y) return SPH_ERR_ARG;
    int64_t o = 0;
    for (int s = 0; s < cfg->nstart; s++) {
        const sph_rect_spawner &sp = cfg->start[s];
        SplitMix64 r(12345678);  // reseeded per spawner, as sim/config-parser.go:63
        const int64_t o0 = o;
        for (int64_t i = 0; i < sp.n; i++, o++) {
            x[o] = sp.upper_left[0] + r.uni() * (sp.lower_right[0] - sp.upper_left[0]);
            y[o] = sp.upper_left[1] + r.uni() * (sp.lower_right[1] - sp.upper_left[1]);
            if (vx) vx[o] = 0.0;
            if (vy) vy[o] = 0.0;
            if (u) u[o] = 0.01;
        }
        // then Z = rand.Int() per particle (a second pass, as sim/config-parser.go:73-76)
        for (int64_t i = 0; i < sp.n; i++) {
            const int64_t zi = (int64_t)(r.next() >> 1);
            if (z) z[o0 + i] = zi;
        }
    }
    return SPH_OK;
}

int64_t sph_point_source_spawn(sph_point_source *src, double t, uint64_t seed, double *x, double *y, double *vx,
                               double *vy, double *u, int64_t *z) {
    if (!src || !(src->rate > 0)) return 0;
    const double dt = t - src->last_spawned;
    const double cooldown = 1.0 / src->rate;
    const int64_t n = (int64_t)(dt / cooldown);
    if (n <= 0) return 0;
    src->last_spawned += (double)n * cooldown;
    if (x && y) {
        SplitMix64 r(seed);
        for (int64_t i = 0; i < n; i++) {
            const double dy = 0.01 * (-1.0 + 2.0 * r.uni());
            const double dx = 0.01 * (-1.0 + 2.0 * r.uni());
            const int64_t zi = (int64_t)(r.next() >> 1);  // Z = rand.Int()
            x[i] = src->origin[0] + dx;
            y[i] = src->origin[1] + dy;
            if (vx) vx[i] = 0.0;
            if (vy) vy[i] = 0.0;
            if (u) u[i] = 0.002;
            if (z) z[i] = zi;
        }
    }
    return n;
}

}  // extern "C"

namespace sphgpu {

// gx.ParaRamp (gx/graphics.go:156-164) for every index, in FP64 without
// contraction (this file is compiled with -ffp-contract=off), as NRGBA bytes.
void para_ramp_table(unsigned char out[256 * 4]) {
    for (int i = 0; i < 256; i++) {
        const double x = (double)i;
        const double r = std::fmin(215.0, std::fmax(0.0, -std::fabs((x - 60) * 31 / 17 - 232) + 245));
        const double g = std::fmin(190.0, std::fmax(0.0, -std::fabs(x * 31 / 17 - 232) + 245));
        const double b = std::fmin(215.0, std::fmax(0.0, -std::fabs((x + 70) * 31 / 17 - 232) + 245));
        out[4 * i + 0] = (unsigned char)r;
        out[4 * i + 1] = (unsigned char)g;
        out[4 * i + 2] = (unsigned char)b;
        out[4 * i + 3] = 255;
    }
}

}  // namespace sphgpu
