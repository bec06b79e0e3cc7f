// Parameter parsing: a small JSON reader (nlohmann-json is not available) and
// the mapping of the reference's GPUHybrid keys (GPUHybrid.cu:106-179) plus
// this implementation's "gb300" extension object.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <map>
#include <memory>

#include "lss_common.hpp"

namespace lss {
namespace {

struct JValue {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0;
    std::string str;
    std::vector<JValue> arr;
    std::map<std::string, JValue> obj;
};

struct JParser {
    const char *s;
    size_t i = 0;
    explicit JParser(const char *t) : s(t) {}

    [[noreturn]] void bad(const std::string &m)
    {
        fail(LSS_ERR_INVALID_ARGUMENT, "parameter JSON: " + m + " at offset " + std::to_string(i));
    }
    void ws()
    {
        while (s[i] && std::isspace((unsigned char)s[i])) ++i;
    }
    bool lit(const char *w)
    {
        size_t k = 0;
        while (w[k] && s[i + k] == w[k]) ++k;
        if (w[k]) return false;
        i += k;
        return true;
    }
    JValue parse()
    {
        ws();
        JValue v;
        char c = s[i];
        if (c == '{') {
            v.kind = JValue::Obj;
            ++i;
            ws();
            if (s[i] == '}') { ++i; return v; }
            for (;;) {
                ws();
                if (s[i] != '"') bad("expected key");
                std::string k = str();
                ws();
                if (s[i] != ':') bad("expected ':'");
                ++i;
                v.obj[k] = parse();
                ws();
                if (s[i] == ',') { ++i; continue; }
                if (s[i] == '}') { ++i; break; }
                bad("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.kind = JValue::Arr;
            ++i;
            ws();
            if (s[i] == ']') { ++i; return v; }
            for (;;) {
                v.arr.push_back(parse());
                ws();
                if (s[i] == ',') { ++i; continue; }
                if (s[i] == ']') { ++i; break; }
                bad("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.kind = JValue::Str;
            v.str = str();
        } else if (lit("true")) {
            v.kind = JValue::Bool; v.b = true;
        } else if (lit("false")) {
            v.kind = JValue::Bool; v.b = false;
        } else if (lit("null")) {
            v.kind = JValue::Null;
        } else {
            char *end = nullptr;
            double d = std::strtod(s + i, &end);
            if (end == s + i) bad("unexpected character");
            i = (size_t)(end - s);
            v.kind = JValue::Num;
            v.num = d;
        }
        return v;
    }
    std::string str()
    {
        ++i;  // opening quote
        std::string out;
        while (s[i] && s[i] != '"') {
            if (s[i] == '\\') {
                ++i;
                char e = s[i];
                if (e == 'n') out += '\n';
                else if (e == 't') out += '\t';
                else if (e == 'u') { out += '?'; i += 4; }
                else out += e;
                ++i;
            } else {
                out += s[i++];
            }
        }
        if (s[i] != '"') bad("unterminated string");
        ++i;
        return out;
    }
};

double num(const JValue &v, const char *key)
{
    if (v.kind == JValue::Num) return v.num;
    if (v.kind == JValue::Bool) return v.b ? 1.0 : 0.0;
    fail(LSS_ERR_INVALID_ARGUMENT, std::string("parameter ") + key + " must be a number");
}
bool boolean(const JValue &v, const char *key)
{
    if (v.kind == JValue::Bool) return v.b;
    if (v.kind == JValue::Num) return v.num != 0.0;
    fail(LSS_ERR_INVALID_ARGUMENT, std::string("parameter ") + key + " must be a boolean");
}
int integer(const JValue &v, const char *key)
{
    double d = num(v, key);
    if (d > 2147483647.0) d = 2147483647.0;
    if (d < -2147483648.0) d = -2147483648.0;
    return (int)d;
}

}  // namespace

Params parse_params(const char *json, const Params &base)
{
    Params p = base;
    if (!json || !*json) return p;
    JParser jp(json);
    JValue root = jp.parse();
    if (root.kind != JValue::Obj) fail(LSS_ERR_INVALID_ARGUMENT, "parameter JSON must be an object");
    if (root.obj.count("solver")) {
        const JValue &sv = root.obj.at("solver");
        std::string name = sv.kind == JValue::Str ? sv.str
                           : (sv.kind == JValue::Arr && !sv.arr.empty() && sv.arr[0].kind == JValue::Str)
                               ? sv.arr[0].str
                               : std::string();
        if (!name.empty() && name != "GPUHybrid" && name != "GPUHybridSolver")
            fail(LSS_ERR_UNSUPPORTED, "solver \"" + name + "\" is not provided by this library");
    }
    const JValue *g = nullptr;
    if (root.obj.count("GPUHybrid")) g = &root.obj.at("GPUHybrid");
    else if (root.obj.count("GPUHybridSolver")) g = &root.obj.at("GPUHybridSolver");
    if (g && g->kind == JValue::Obj) {
        for (const auto &kv : g->obj) {
            const std::string &k = kv.first;
            const JValue &v = kv.second;
            const char *kc = k.c_str();
            if (k == "max_iter") p.max_iter = integer(v, kc);
            else if (k == "relative_tolerance") p.rel_tol = num(v, kc);
            else if (k == "absolute_tolerance") p.abs_tol = num(v, kc);
            else if (k == "theta") p.theta = num(v, kc);
            else if (k == "select_bad_dofs_from_l1_norm") p.select_l1 = boolean(v, kc);
            else if (k == "block_size") p.block_size = integer(v, kc);
            else if (k == "do_hybrid_precond") p.do_hybrid = boolean(v, kc);
            else if (k == "decompose_subdomains") p.decompose = boolean(v, kc);
            else if (k == "min_subdomain_size") p.min_sub = integer(v, kc);
            else if (k == "max_subdomain_size") p.max_sub = integer(v, kc);
            else if (k == "max_dense_size") p.max_dense_size = integer(v, kc);
            else if (k == "gmm_jump_threshold") p.jump_threshold = num(v, kc);
            else if (k == "expand_subdomains") p.expand = boolean(v, kc);
            else if (k == "use_float_on_subdomains") p.float_subdomains = boolean(v, kc);
            else if (k == "gmm_tol") p.gmm_tol = num(v, kc);
            else if (k == "max_gmm_iterations") p.max_gmm_iterations = integer(v, kc);
            else if (k == "conditioning_threshold") p.cond_threshold = num(v, kc);
            // unknown keys are ignored, as the reference's set_parameters does
        }
    }
    if (root.obj.count("gb300") && root.obj.at("gb300").kind == JValue::Obj) {
        for (const auto &kv : root.obj.at("gb300").obj) {
            const std::string &k = kv.first;
            const JValue &v = kv.second;
            const char *kc = k.c_str();
            if (k == "precision") {
                if (v.kind != JValue::Str || (v.str != "fp64" && v.str != "mixed"))
                    fail(LSS_ERR_INVALID_ARGUMENT, "gb300.precision must be \"fp64\" or \"mixed\"");
                p.mixed = v.str == "mixed";
            } else if (k == "precond_residual") {
                if (v.kind != JValue::Str || (v.str != "auto" && v.str != "fp32" && v.str != "df32"))
                    fail(LSS_ERR_INVALID_ARGUMENT,
                         "gb300.precond_residual must be \"auto\", \"fp32\" or \"df32\"");
                p.precond_residual = v.str == "auto" ? 0 : (v.str == "fp32" ? 1 : 2);
            } else if (k == "mas_offdiag") {
                if (v.kind != JValue::Str || (v.str != "fp32" && v.str != "bf16"))
                    fail(LSS_ERR_INVALID_ARGUMENT, "gb300.mas_offdiag must be \"fp32\" or \"bf16\"");
                p.mas_bf16_offdiag = v.str == "bf16";
            } else if (k == "bad_dof_strategy") {
                if (v.kind != JValue::Str ||
                    (v.str != "gpuhybrid" && v.str != "elbow" && v.str != "kmean" && v.str != "gmm"))
                    fail(LSS_ERR_INVALID_ARGUMENT,
                         "gb300.bad_dof_strategy must be \"gpuhybrid\", \"elbow\", \"kmean\" or \"gmm\"");
                p.bad_dof_strategy = v.str == "gpuhybrid" ? 0 : (v.str == "elbow" ? 1 : (v.str == "kmean" ? 2 : 3));
            } else if (k == "bad_dof_kmeans_search_fraction") {
                p.kmeans_search_fraction = num(v, kc);
            } else if (k == "bad_dof_kmeans_jump_threshold") {
                p.kmeans_jump_threshold = num(v, kc);
            } else if (k == "bad_dof_kmeans_max_iterations") {
                p.kmeans_max_iterations = integer(v, kc);
            } else if (k == "bad_dof_kmeans_expand_neighbors") {
                p.kmeans_expand_neighbors = integer(v, kc);
            } else if (k == "bad_dof_gmm_jump_threshold") {
                p.mas_gmm_jump_threshold = num(v, kc);
            } else if (k == "bad_dof_gmm_tol") {
                p.mas_gmm_tol = num(v, kc);
            } else if (k == "bad_dof_gmm_max_iterations") {
                p.mas_gmm_max_iterations = integer(v, kc);
            } else if (k == "bad_dof_gmm_expand_neighbors") {
                p.mas_gmm_expand_neighbors = integer(v, kc);
            } else if (k == "bad_dof_max_block") {
                p.bad_dof_max_block = integer(v, kc);
            } else if (k == "outer_spmv") {
                if (v.kind != JValue::Str || (v.str != "auto" && v.str != "fp64" && v.str != "df32"))
                    fail(LSS_ERR_INVALID_ARGUMENT, "gb300.outer_spmv must be \"auto\", \"fp64\" or \"df32\"");
                p.outer_spmv = v.str == "auto" ? 0 : (v.str == "fp64" ? 1 : 2);
            } else if (k == "composition") {
                if (v.kind != JValue::Str || (v.str != "multiplicative" && v.str != "additive"))
                    fail(LSS_ERR_INVALID_ARGUMENT,
                         "gb300.composition must be \"multiplicative\" or \"additive\"");
                p.multiplicative = v.str == "multiplicative";
            } else if (k == "max_coarse_levels") p.max_coarse_levels = integer(v, kc);
            else if (k == "mas_damping") p.mas_damping = num(v, kc);
            else if (k == "omega_iters") p.omega_iters = integer(v, kc);
            else if (k == "omega_factor") p.omega_factor = num(v, kc);
            else if (k == "check_every") p.check_every = integer(v, kc);
            else if (k == "max_refinements") p.max_refinements = integer(v, kc);
            else if (k == "device") p.device = integer(v, kc);
            else if (k == "partition_threads") p.partition_threads = integer(v, kc);
            else if (k == "use_graphs") p.use_graphs = boolean(v, kc);
            else if (k == "spmv_lanes") p.spmv_lanes = integer(v, kc);
            else if (k == "memory_cap_bytes") p.memory_cap_bytes = (size_t)num(v, kc);
            else fail(LSS_ERR_INVALID_ARGUMENT, "unknown gb300 parameter \"" + k + "\"");
        }
    }
    if (p.block_size < 1 || p.block_size > 3)
        fail(LSS_ERR_INVALID_ARGUMENT, "block_size must be 1, 2 or 3");
    if (p.max_coarse_levels < 1 || p.max_coarse_levels > 6)
        fail(LSS_ERR_INVALID_ARGUMENT, "gb300.max_coarse_levels must be in [1, 6]");
    if (p.check_every < 1) p.check_every = 1;
    if (!(p.kmeans_search_fraction > 0.0) || p.kmeans_search_fraction > 1.0)
        fail(LSS_ERR_INVALID_ARGUMENT, "gb300.bad_dof_kmeans_search_fraction must be in (0, 1]");
    if (p.spmv_lanes != 0 && (p.spmv_lanes < 1 || p.spmv_lanes > 32 || (p.spmv_lanes & (p.spmv_lanes - 1))))
        fail(LSS_ERR_INVALID_ARGUMENT, "gb300.spmv_lanes must be 0 (autotune) or a power of two <= 32");
    if (p.omega_iters < 1 || p.omega_iters > 64) fail(LSS_ERR_INVALID_ARGUMENT, "gb300.omega_iters must be in [1, 64]");
    if (!(p.omega_factor > 0.0) || p.omega_factor >= 2.0)
        fail(LSS_ERR_INVALID_ARGUMENT, "gb300.omega_factor must be in (0, 2)");
    if (p.max_iter < 0) p.max_iter = 0;
    return p;
}

}  // namespace lss
