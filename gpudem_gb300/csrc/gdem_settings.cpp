// demSettings.json, the particle file of the "file" inlet and ASCII STL
// walls, read on the host the way the reference's main program reads them
// (main.cu:44-140, settings_loader.cu, ParticleSystem.cu:189-440,
// TriangleMesh.cu:347-560), with the gaps that stop the shipped cases closed:
//
//  * particleTypes.particle0.YoungModulus (main.cu:64) is optional: every
//    shipped case gives the stiffness "k" instead, which is then used as is
//    (the reference derives k from E, ParticleSystem.cu:202);
//  * others.bruteOn (main.cu:72) is optional, 0 by default;
//  * inlet.file is accepted as the file name itself (what the shipped cases
//    hold) or as an object {"name": ...}.  The reference's string getter
//    accepts only objects (cJSON_d.c:3226-3232), so its file inlet could
//    never start.
//
// Missing or mistyped keys return GDEM_ERR_ARG with the key's path in the
// message, where the reference abort()s.  Derived constants (mass,
// stiffness, damping constant, time step) follow the reference's operation
// order; this unit compiles without floating-point contraction.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "gdem.h"

namespace {

constexpr double kPiRef = 3.14159265359;  // PI, hardCodedParameters.h:6

// ---------------------------------------------------------------- JSON
struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    double num = 0.;
    bool b = false;
    std::string str;
    std::vector<std::unique_ptr<JValue>> arr;
    std::vector<std::pair<std::string, std::unique_ptr<JValue>>> obj;  // file order

    const JValue* get(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return kv.second.get();
        return nullptr;
    }
};

// Recursive-descent parser of RFC 8259 JSON (numbers by strtod, \uXXXX
// escapes kept to the basic plane).
struct JParser {
    const char* p;
    const char* end;
    std::string err;
    int depth = 0;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    bool fail(const char* what) {
        if (err.empty()) err = what;
        return false;
    }
    bool lit(const char* s) {
        const size_t n = strlen(s);
        if ((size_t)(end - p) < n || strncmp(p, s, n) != 0) return false;
        p += n;
        return true;
    }
    bool string(std::string& out) {
        if (p >= end || *p != '"') return fail("expected a string");
        p++;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c == '\\') {
                if (p >= end) return fail("bad escape");
                const char e = *p++;
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
                        if (end - p < 4) return fail("bad \\u escape");
                        unsigned cp = 0;
                        for (int k = 0; k < 4; k++) {
                            const char h = *p++;
                            cp <<= 4;
                            if (h >= '0' && h <= '9') cp |= (unsigned)(h - '0');
                            else if (h >= 'a' && h <= 'f') cp |= (unsigned)(h - 'a' + 10);
                            else if (h >= 'A' && h <= 'F') cp |= (unsigned)(h - 'A' + 10);
                            else return fail("bad \\u escape");
                        }
                        if (cp < 0x80) {
                            out += (char)cp;
                        } else if (cp < 0x800) {
                            out += (char)(0xC0 | (cp >> 6));
                            out += (char)(0x80 | (cp & 0x3F));
                        } else {
                            out += (char)(0xE0 | (cp >> 12));
                            out += (char)(0x80 | ((cp >> 6) & 0x3F));
                            out += (char)(0x80 | (cp & 0x3F));
                        }
                        break;
                    }
                    default: return fail("bad escape");
                }
            } else {
                out += c;
            }
        }
        if (p >= end) return fail("unterminated string");
        p++;
        return true;
    }
    bool value(JValue& v) {
        if (++depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        bool ok = true;
        if (*p == '{') {
            v.kind = JValue::Object;
            p++;
            ws();
            if (p < end && *p == '}') {
                p++;
            } else {
                for (;;) {
                    ws();
                    std::string key;
                    if (!string(key)) return false;
                    ws();
                    if (p >= end || *p != ':') return fail("expected ':'");
                    p++;
                    auto child = std::make_unique<JValue>();
                    if (!value(*child)) return false;
                    v.obj.emplace_back(std::move(key), std::move(child));
                    ws();
                    if (p < end && *p == ',') { p++; continue; }
                    if (p < end && *p == '}') { p++; break; }
                    return fail("expected ',' or '}'");
                }
            }
        } else if (*p == '[') {
            v.kind = JValue::Array;
            p++;
            ws();
            if (p < end && *p == ']') {
                p++;
            } else {
                for (;;) {
                    auto child = std::make_unique<JValue>();
                    if (!value(*child)) return false;
                    v.arr.push_back(std::move(child));
                    ws();
                    if (p < end && *p == ',') { p++; continue; }
                    if (p < end && *p == ']') { p++; break; }
                    return fail("expected ',' or ']'");
                }
            }
        } else if (*p == '"') {
            v.kind = JValue::String;
            ok = string(v.str);
        } else if (lit("true")) {
            v.kind = JValue::Bool;
            v.b = true;
        } else if (lit("false")) {
            v.kind = JValue::Bool;
        } else if (lit("null")) {
            v.kind = JValue::Null;
        } else {
            // a number: JSON grammar checked loosely, value by strtod
            const char* q = p;
            if (q < end && *q == '-') q++;
            if (q >= end || !(*q >= '0' && *q <= '9')) return fail("unexpected character");
            std::string tok;
            while (p < end && (strchr("+-0123456789.eE", *p) != nullptr)) tok += *p++;
            char* e2 = nullptr;
            v.kind = JValue::Number;
            v.num = strtod(tok.c_str(), &e2);
            if (!e2 || *e2 != '\0') return fail("bad number");
        }
        depth--;
        return ok;
    }
};

// ---------------------------------------------------------------- settings
struct Reader {
    std::string err;
    const JValue* obj(const JValue* parent, const char* key, const char* path) {
        const JValue* v = parent ? parent->get(key) : nullptr;
        if (!v || v->kind != JValue::Object) {
            if (err.empty()) err = std::string("missing or not an object: ") + path;
            return nullptr;
        }
        return v;
    }
    double num(const JValue* parent, const char* key, const char* path, bool required = true, double dflt = NAN) {
        const JValue* v = parent ? parent->get(key) : nullptr;
        if (!v) {
            if (required && err.empty()) err = std::string("missing number: ") + path;
            return dflt;
        }
        if (v->kind != JValue::Number) {
            if (err.empty()) err = std::string("not a number: ") + path;
            return dflt;
        }
        return v->num;
    }
    // cJSON's valueint: the double saturated to the int range, then truncated
    int integer(const JValue* parent, const char* key, const char* path, bool required = true, int dflt = 0) {
        const double d = num(parent, key, path, required, (double)dflt);
        if (d != d) return dflt;
        if (d >= 2147483647.) return 2147483647;
        if (d <= -2147483648.) return (-2147483647 - 1);
        return (int)d;
    }
};

void put_msg(char* msg, int len, const std::string& s) {
    if (msg && len > 0) {
        strncpy(msg, s.c_str(), (size_t)len - 1);
        msg[len - 1] = '\0';
    }
}

bool copy_path(char* dst, const std::string& s) {
    if (s.size() >= GDEM_SETTINGS_PATH) return false;
    memcpy(dst, s.c_str(), s.size() + 1);
    return true;
}

int parse_settings(const std::string& text, gdem_settings* s, std::string& err) {
    JParser P{text.data(), text.data() + text.size(), {}};
    JValue root;
    if (!P.value(root)) {
        err = "JSON: " + P.err + " at byte " + std::to_string(P.p - text.data());
        return GDEM_ERR_ARG;
    }
    P.ws();
    if (P.p != P.end) {
        err = "JSON: trailing characters at byte " + std::to_string(P.p - text.data());
        return GDEM_ERR_ARG;
    }
    if (root.kind != JValue::Object) {
        err = "JSON: the settings must be an object";
        return GDEM_ERR_ARG;
    }
    memset(s, 0, sizeof(*s));
    Reader R;
    // particleTypes.particle0 (main.cu:54-64)
    const JValue* types = R.obj(&root, "particleTypes", "particleTypes");
    const JValue* p0 = R.obj(types, "particle0", "particleTypes.particle0");
    s->radius = R.num(p0, "radius", "particleTypes.particle0.radius");
    s->restitution = R.num(p0, "CoR", "particleTypes.particle0.CoR");
    s->density = R.num(p0, "density", "particleTypes.particle0.density");
    s->mu = R.num(p0, "mu", "particleTypes.particle0.mu");
    s->youngs_modulus = R.num(p0, "YoungModulus", "particleTypes.particle0.YoungModulus", false);
    s->k_given = R.num(p0, "k", "particleTypes.particle0.k", false);
    if (R.err.empty() && s->youngs_modulus != s->youngs_modulus && s->k_given != s->k_given)
        R.err = "particleTypes.particle0 needs YoungModulus or k";
    // others (main.cu:68-72, 123-126)
    const JValue* others = R.obj(&root, "others", "others");
    s->gpu_on = R.integer(others, "gpuOn", "others.gpuOn");
    s->brute_on = R.integer(others, "bruteOn", "others.bruteOn", false, 0);
    s->seed = R.integer(others, "seed", "others.seed", false, 1);
    s->dt_factor = R.num(others, "dtFactor", "others.dtFactor");
    s->start_time = R.num(others, "startTime", "others.startTime", false, 0.);
    s->end_time = R.num(others, "endTime", "others.endTime");
    s->output_timing = R.num(others, "outputTiming", "others.outputTiming");
    // gravity (main.cu:115-119)
    const JValue* grav = R.obj(&root, "gravity", "gravity");
    s->g[0] = R.num(grav, "x", "gravity.x");
    s->g[1] = R.num(grav, "y", "gravity.y");
    s->g[2] = R.num(grav, "z", "gravity.z");
    // walls.filepaths (main.cu:76, 94; load_ascii_stl_double, TriangleMesh.cu:363-386)
    const JValue* walls = R.obj(&root, "walls", "walls");
    const JValue* files = walls ? walls->get("filepaths") : nullptr;
    if (R.err.empty()) {
        if (!files || files->kind != JValue::Array) {
            R.err = "missing or not an array: walls.filepaths";
        } else if (files->arr.size() > GDEM_SETTINGS_MAX_WALLS) {
            R.err = "more than GDEM_SETTINGS_MAX_WALLS wall files";
        } else {
            for (const auto& f : files->arr) {
                if (f->kind != JValue::String) {
                    R.err = "walls.filepaths: not a string";
                    break;
                }
                if (!copy_path(s->walls[s->n_walls++], f->str)) {
                    R.err = "walls.filepaths: path too long";
                    break;
                }
            }
        }
    }
    // inlet (main.cu:80, 131-133; ParticleSystem.cu:205-360)
    const JValue* inlet = R.obj(&root, "inlet", "inlet");
    s->n_particles = R.integer(inlet, "numParticle", "inlet.numParticle");
    if (R.err.empty() && s->n_particles <= 0) R.err = "inlet.numParticle must be positive";
    const JValue* mode = inlet ? inlet->get("inputMode") : nullptr;
    if (R.err.empty()) {
        if (!mode || mode->kind != JValue::String) {
            R.err = "missing or not a string: inlet.inputMode";
        } else if (mode->str == "shuffle") {
            s->input_mode = GDEM_INLET_SHUFFLE;
            const JValue* sh = R.obj(inlet, "shuffle", "inlet.shuffle");
            const char* lo[3] = {"minx", "miny", "minz"};
            const char* hi[3] = {"maxx", "maxy", "maxz"};
            for (int a = 0; a < 3; a++) {
                s->inlet_min[a] = R.num(sh, lo[a], (std::string("inlet.shuffle.") + lo[a]).c_str());
                s->inlet_max[a] = R.num(sh, hi[a], (std::string("inlet.shuffle.") + hi[a]).c_str());
            }
        } else if (mode->str == "file") {
            s->input_mode = GDEM_INLET_FILE;
            const JValue* f = inlet->get("file");
            const JValue* name = nullptr;
            if (f && f->kind == JValue::String) name = f;
            else if (f && f->kind == JValue::Object) name = f->get("name");
            if (!name || name->kind != JValue::String)
                R.err = "inlet.file: needs the file name (a string, or an object with \"name\")";
            else if (!copy_path(s->particle_file, name->str))
                R.err = "inlet.file: path too long";
            // the region is the particles' bounding box (ParticleSystem.cu:392-440),
            // known once gdem_read_particle_file has read them
            for (int a = 0; a < 3; a++) {
                s->inlet_min[a] = NAN;
                s->inlet_max[a] = NAN;
            }
        } else {
            R.err = "inlet.inputMode: neither \"shuffle\" nor \"file\"";
        }
    }
    if (!R.err.empty()) {
        err = R.err;
        return GDEM_ERR_ARG;
    }
    if (!(s->radius > 0) || !(s->density > 0) || !(s->restitution > 0 && s->restitution <= 1) || !(s->mu >= 0) ||
        !(s->dt_factor > 0) || !(s->output_timing > 0)) {
        err = "radius, density, dtFactor and outputTiming must be positive, CoR in (0, 1], mu >= 0";
        return GDEM_ERR_ARG;
    }
    // derived constants, in the reference's operation order
    const double r = s->radius;
    s->mass = s->density * 3.14 * r * r * r * 4. / 3.;  // main.cu:67
    if (s->youngs_modulus == s->youngs_modulus) {
        const double E = s->youngs_modulus;
        s->stiffness = 4. / 3. * (E * 0.5) * sqrt(r * 0.5) * sqrt(0.05 * r);  // ParticleSystem.cu:202
    } else {
        s->stiffness = s->k_given;
    }
    if (!(s->stiffness > 0)) {
        err = "the stiffness (k, or from YoungModulus) must be positive";
        return GDEM_ERR_ARG;
    }
    const double res = s->restitution;
    s->etaconst = -2. * log(res) * sqrt(s->stiffness / (3.1415 * 3.1415 + log(res) * log(res)));  // ParticleSystem.cu:301
    // main.cu:123-129: dt from the contact time, snapped so that the output
    // interval is a whole number of steps
    const double dt0 = 2. * kPiRef * sqrt(s->mass / s->stiffness) / s->dt_factor;
    s->out_step = (int)floor(s->output_timing / dt0);
    if (s->out_step < 1) {
        err = "outputTiming is shorter than one time step";
        return GDEM_ERR_ARG;
    }
    s->dt = s->output_timing / (double)s->out_step;
    return GDEM_OK;
}

bool read_file(const char* path, std::string& out) {
    FILE* fp = fopen(path, "rb");
    if (!fp) return false;
    char buf[65536];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), fp)) > 0) out.append(buf, got);
    const bool ok = !ferror(fp);
    fclose(fp);
    return ok;
}

}  // namespace

extern "C" {

int gdem_settings_parse(const char* json_text, gdem_settings* s, char* msg, int msg_len) {
    if (!json_text || !s) {
        put_msg(msg, msg_len, "null argument");
        return GDEM_ERR_ARG;
    }
    std::string err;
    const int rc = parse_settings(std::string(json_text), s, err);
    put_msg(msg, msg_len, err);
    return rc;
}

int gdem_settings_load(const char* path, gdem_settings* s, char* msg, int msg_len) {
    if (!path || !s) {
        put_msg(msg, msg_len, "null argument");
        return GDEM_ERR_ARG;
    }
    std::string text;
    if (!read_file(path, text)) {
        put_msg(msg, msg_len, std::string("cannot read ") + path);
        return GDEM_ERR_ARG;
    }
    std::string err;
    const int rc = parse_settings(text, s, err);
    put_msg(msg, msg_len, err);
    return rc;
}

// The "file" inlet's particle file (ParticleSystem.cu:357-440): a CSV with a
// header line naming the columns x, y, z, vx, vy, vz (in any order, other
// columns ignored), then one particle per line.  Exactly n data lines.
int gdem_read_particle_file(const char* path, int n, double* x, double* v, double* box_min, double* box_max) {
    if (!path || n <= 0 || !x) return GDEM_ERR_ARG;
    std::string text;
    if (!read_file(path, text)) return GDEM_ERR_ARG;
    std::vector<std::string> lines;
    size_t a = 0;
    while (a < text.size()) {
        size_t b = text.find('\n', a);
        if (b == std::string::npos) b = text.size();
        std::string ln = text.substr(a, b - a);
        if (!ln.empty() && ln.back() == '\r') ln.pop_back();
        if (!ln.empty()) lines.push_back(ln);
        a = b + 1;
    }
    if (lines.size() != (size_t)n + 1) return GDEM_ERR_ARG;  // header + n rows
    auto split = [](const std::string& ln) {
        std::vector<std::string> out;
        size_t s0 = 0;
        for (;;) {
            const size_t c = ln.find(',', s0);
            std::string f = ln.substr(s0, c == std::string::npos ? std::string::npos : c - s0);
            const size_t i0 = f.find_first_not_of(" \t"), i1 = f.find_last_not_of(" \t");
            out.push_back(i0 == std::string::npos ? std::string() : f.substr(i0, i1 - i0 + 1));
            if (c == std::string::npos) break;
            s0 = c + 1;
        }
        return out;
    };
    const std::vector<std::string> head = split(lines[0]);
    const char* want[6] = {"x", "y", "z", "vx", "vy", "vz"};
    int col[6];
    for (int k = 0; k < 6; k++) {
        col[k] = -1;
        for (size_t c = 0; c < head.size(); c++)
            if (head[c] == want[k]) col[k] = (int)c;
        if (col[k] < 0) return GDEM_ERR_ARG;
    }
    double lo[3] = {1.e16, 1.e16, 1.e16}, hi[3] = {-1.e16, -1.e16, -1.e16};
    for (int i = 0; i < n; i++) {
        const std::vector<std::string> f = split(lines[(size_t)i + 1]);
        double val[6];
        for (int k = 0; k < 6; k++) {
            if ((size_t)col[k] >= f.size() || f[(size_t)col[k]].empty()) return GDEM_ERR_ARG;
            char* e = nullptr;
            val[k] = strtod(f[(size_t)col[k]].c_str(), &e);
            if (!e || *e != '\0') return GDEM_ERR_ARG;
        }
        for (int k = 0; k < 3; k++) {
            x[3 * i + k] = val[k];
            if (v) v[3 * i + k] = val[3 + k];
            if (hi[k] < val[k]) hi[k] = val[k];
            if (lo[k] > val[k]) lo[k] = val[k];
        }
    }
    for (int k = 0; k < 3; k++) {
        if (box_min) box_min[k] = lo[k];
        if (box_max) box_max[k] = hi[k];
    }
    return GDEM_OK;
}

// Triangles of an ASCII STL file in file order, as load_ascii_stl_double
// reads them (TriangleMesh.cu:347-386, 483-533): a facet starts at a line
// "facet normal ..." (after any whitespace); its three vertex lines follow
// the "outer loop" line.  tris receives 9 doubles per triangle (up to cap
// triangles); the return value is the file's triangle count, or -1 when it
// cannot be read or a facet is cut short.
int gdem_read_stl(const char* path, double* tris, int cap) {
    if (!path || cap < 0) return -1;
    FILE* fp = fopen(path, "r");
    if (!fp) return -1;
    char line[256];
    int count = 0;
    bool bad = false;
    while (fgets(line, sizeof(line), fp)) {
        double nx, ny, nz;
        if (sscanf(line, " facet normal %lf %lf %lf", &nx, &ny, &nz) != 3) continue;
        if (!fgets(line, sizeof(line), fp)) { bad = true; break; }  // outer loop
        for (int c = 0; c < 3; c++) {
            double x, y, z;
            if (!fgets(line, sizeof(line), fp) || sscanf(line, " vertex %lf %lf %lf", &x, &y, &z) != 3) {
                bad = true;
                break;
            }
            if (tris && count < cap) {
                tris[9 * (size_t)count + 3 * c] = x;
                tris[9 * (size_t)count + 3 * c + 1] = y;
                tris[9 * (size_t)count + 3 * c + 2] = z;
            }
        }
        if (bad) break;
        count++;
    }
    fclose(fp);
    return bad ? -1 : count;
}

}  // extern "C"
