// gopf_model.cpp -- equation-string front end: the pf.Model / pf.Build
// algebra, compiled into the device term table.
//
// A Go caller can hand the library the same strings it gives pf.Model
// (pf/model.go:157-162) and get the same split into explicit terms (Terms)
// and implicit terms (Denum) that pf.Build makes (pf/rhsBuilder.go:26-54):
//   - SplitOnMany over "+"/"-" with the preceding delimiter as sign
//     (pf/util.go:154-199);
//   - known prefixes "-", "LAP^4", "LAP^2", "LAP", "*" for user-defined terms
//     (pf/rhsBuilder.go:244-297, constructFunc 199-242);
//   - a term bilinear in its own field goes to the denominator with the field
//     name removed (isBilinear 69-106);
//   - otherwise ConcreteTerm (125-190): sign * prod(scalar^p) * brick *
//     LAP^n, where brick is the longest field / derived-field name contained
//     in the term (GetFieldName, pf/util.go:83-104);
//   - non-bilinear field expressions become derived fields named by their
//     sorted factors (UpdateDerivedFields pf/model.go:165-195,
//     GetNonLinearFieldExpressions pf/util.go:17-34, SortFactors 291-296).
// Scalars are evaluated once, as the product of real parts of their powers;
// a complex scalar has no device implementation and is rejected.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "gopf_ctx.h"

namespace {

struct SubDelim {
    std::string sub;
    std::string delim;
};

bool contains(const std::string &s, const std::string &t) { return s.find(t) != std::string::npos; }

std::string replace_all(std::string s, const std::string &from, const std::string &to)
{
    if (from.empty()) return s;
    size_t pos = 0;
    while ((pos = s.find(from, pos)) != std::string::npos) {
        s.replace(pos, from.size(), to);
        pos += to.size();
    }
    return s;
}

std::vector<std::string> split(const std::string &s, char c)
{
    std::vector<std::string> out;
    std::string cur;
    for (char ch : s) {
        if (ch == c) {
            out.push_back(cur);
            cur.clear();
        } else {
            cur += ch;
        }
    }
    out.push_back(cur);
    return out;
}

// pf/util.go:154-199
std::vector<SubDelim> split_on_many(const std::string &value, const std::vector<std::string> &delims)
{
    std::vector<SubDelim> out;
    std::string first;
    if (!value.empty())
        for (auto &d : delims)
            if (value.substr(0, 1) == d) first = d;
    std::vector<SubDelim> queue{{value, first}};
    std::string all;
    for (auto &d : delims) all += d;
    size_t head = 0;
    while (head < queue.size()) {
        SubDelim cur = queue[head++];
        if (cur.sub.find_first_of(all) == std::string::npos) {
            out.push_back(cur);
            continue;
        }
        std::string delim = delims[0];
        for (auto &d : delims)
            if (contains(cur.sub, d)) {
                delim = d;
                break;
            }
        std::vector<std::string> parts = split(cur.sub, delim[0]);
        std::vector<std::string> nonempty;
        for (auto &p : parts)
            if (!p.empty()) nonempty.push_back(p);
        if (nonempty.empty()) continue;
        queue.push_back({nonempty[0], cur.delim});
        for (size_t i = 1; i < nonempty.size(); ++i) queue.push_back({nonempty[i], delim});
    }
    return out;
}

const std::vector<std::string> &known_prefixes()
{
    static const std::vector<std::string> p{"-", "LAP^4", "LAP^2", "LAP", "*"};
    return p;
}

// pf/rhsBuilder.go:267-281
std::vector<std::string> get_known_prefixes(std::string s)
{
    std::vector<std::string> pref;
    size_t i = 0;
    const auto &kp = known_prefixes();
    while (i < kp.size()) {
        const std::string &p = kp[i++];
        if (s.compare(0, p.size(), p) == 0) {
            pref.push_back(p);
            s = s.substr(p.size());
            i = 0;
        }
    }
    return pref;
}

std::string remove_known_prefixes(std::string s)
{
    size_t i = 0;
    const auto &kp = known_prefixes();
    while (i < kp.size()) {
        const std::string &p = kp[i++];
        if (s.compare(0, p.size(), p) == 0) {
            s = s.substr(p.size());
            i = 0;
        }
    }
    return s;
}

// pf/util.go:68-80: first "^number" in the pattern, 1 if none
bool get_power(const std::string &pattern, double &power)
{
    static const std::regex re("\\^(-?\\d+\\.?\\d*)");
    std::smatch m;
    if (!std::regex_search(pattern, m, re)) {
        power = 1.0;
        return true;
    }
    try {
        power = std::stod(m[1].str());
    } catch (...) {
        return false;
    }
    return true;
}

std::string regex_escape(const std::string &s)
{
    static const std::string meta = "\\^$.|?*+()[]{}";
    std::string out;
    for (char c : s) {
        if (meta.find(c) != std::string::npos) out += '\\';
        out += c;
    }
    return out;
}

size_t count_matches(const std::string &s, const std::string &lit)
{
    if (lit.empty()) return 0;
    size_t n = 0, pos = 0;
    while ((pos = s.find(lit, pos)) != std::string::npos) {
        ++n;
        pos += lit.size();
    }
    return n;
}

// pf/rhsBuilder.go:69-106
bool is_bilinear(const std::string &term, const std::string &field, const std::vector<std::string> &names)
{
    if (count_matches(term, field) != 1) return false;
    for (auto &f : names) {
        if (f == field) continue;
        if (contains(term, f)) return false;
    }
    // the reference's pattern is field + "*[^/\*]*" (its last letter may repeat)
    std::string fe = regex_escape(field);
    std::regex re(fe + "*[^/\\*]*");
    std::smatch m;
    std::string res;
    if (std::regex_search(term, m, re)) res = m[0].str();
    static const std::regex rp("\\^(-?\\d+\\.?\\d*)");
    std::smatch mp;
    if (!std::regex_search(res, mp, rp)) return true;
    double p;
    try {
        p = std::stod(mp[1].str());
    } catch (...) {
        return true;
    }
    return std::fabs(p - 1.0) < 1e-10;
}

std::string sort_factors(const std::string &expr)
{
    std::vector<std::string> parts = split(expr, '*');
    std::sort(parts.begin(), parts.end());
    std::string out;
    for (size_t i = 0; i < parts.size(); ++i) {
        if (i) out += "*";
        out += parts[i];
    }
    return out;
}

// pf/util.go:17-34
std::string non_linear_field_expressions(const std::string &pattern, const std::string &field,
                                         const std::vector<std::string> &fields)
{
    std::string expr;
    for (auto &f : fields) {
        if (f == field && is_bilinear(pattern, field, fields)) continue;
        size_t pos = pattern.find(f);
        if (pos == std::string::npos) continue;
        size_t end = pos;
        while (end < pattern.size() && pattern[end] != '*') ++end;
        expr += pattern.substr(pos, end - pos) + "*";
    }
    if (expr.size() > 1) return expr.substr(0, expr.size() - 1);
    return expr;
}

// pf/util.go:83-104
std::string get_field_name(const std::string &term, const std::vector<std::string> &names)
{
    std::string field;
    for (auto &f : names) {
        if (!contains(term, f)) continue;
        std::string without = replace_all(term, f, "");
        bool ok = true;
        for (auto &f1 : names)
            if (contains(without, f1)) {
                ok = false;
                break;
            }
        if (ok && f.size() > field.size()) field = f;
    }
    return field;
}

// all maximal runs of non-'*' characters, as Go's FindAllString("[^\*]*") returns them
std::vector<std::string> star_runs(const std::string &term)
{
    std::vector<std::string> out;
    size_t i = 0;
    bool prev_nonempty_end = false;
    size_t prev_end = 0;
    while (i <= term.size()) {
        size_t j = i;
        while (j < term.size() && term[j] != '*') ++j;
        if (j > i) {
            out.push_back(term.substr(i, j - i));
            prev_nonempty_end = true;
            prev_end = j;
            i = j;
            continue;
        }
        // empty match at i: ignored when it abuts the preceding match
        if (!(prev_nonempty_end && prev_end == i)) out.push_back("");
        prev_nonempty_end = false;
        ++i;
    }
    return out;
}

struct Ctx {
    gopf_ctx *ctx;
    gopf_modeldef &d;
    std::vector<std::string> all_field_names() const
    {
        std::vector<std::string> n = d.fields;
        n.insert(n.end(), d.derived_names.begin(), d.derived_names.end());
        return n;
    }
    bool is_field_name(const std::string &n) const
    {
        auto a = all_field_names();
        return std::find(a.begin(), a.end(), n) != a.end();
    }
    bool is_scalar(const std::string &n) const { return d.scalars.count(n) > 0; }
    bool is_brick(const std::string &n) const { return is_scalar(n) || is_field_name(n); }
    bool valid_name(const std::string &name) const
    {
        if (name.empty() || name == "LAP") return true;
        std::string s = name;
        if (s.compare(0, 3, "LAP") == 0) s = s.substr(3);
        return is_brick(s);
    }
    int user_term(const std::string &name, int &kind) const
    {
        for (size_t i = 0; i < d.noise.size(); ++i)
            if (d.noise[i].kind == 2 && d.noise[i].name == name) {
                kind = 3;
                return (int)i;
            }
        for (size_t i = 0; i < d.elastic.size(); ++i)
            if (d.elastic[i].name == name) {
                kind = 1;
                return (int)i;
            }
        for (size_t i = 0; i < d.volcons.size(); ++i)
            if (d.volcons[i].name == name) {
                kind = 2;
                return (int)i;
            }
        for (size_t i = 0; i < d.isym.size(); ++i)
            if (d.isym[i].name == name) {
                kind = 4; // implicit user term: its symbol joins the denominator (pf/rhsBuilder.go:39-40)
                return (int)i;
            }
        return -1;
    }
};

int parse_fail(gopf_ctx *ctx, const std::string &msg) { return gopf_fail(ctx, GOPF_ERR_PARSE, msg); }

bool field_from_leibniz(const std::string &lhs, std::string &field)
{
    if (lhs.size() <= 3) return false;
    if (lhs[0] != 'd' || lhs.substr(lhs.size() - 3) != "/dt") return false;
    field = lhs.substr(1, lhs.size() - 4);
    return true;
}

// register the derived field named by a sorted product description (pf/util.go:38-65)
int add_product_derived(Ctx &c, const std::string &desc)
{
    gopf_derived dv;
    memset(&dv, 0, sizeof(dv));
    dv.kind = GOPF_DER_PRODUCT;
    for (auto &fac : split(desc, '*')) {
        std::string name = fac.substr(0, fac.find('^'));
        int fid = -1;
        for (size_t i = 0; i < c.d.fields.size(); ++i)
            if (c.d.fields[i] == name) fid = (int)i;
        double p;
        if (fid < 0 || !get_power(fac, p)) return parse_fail(c.ctx, "cannot build derived field '" + desc + "'");
        if (dv.nfac >= GOPF_MAX_FACTORS) return parse_fail(c.ctx, "derived field '" + desc + "' has too many factors");
        dv.field[dv.nfac] = fid;
        dv.power[dv.nfac] = (int)std::lround(p);
        dv.coef[dv.nfac] = 1.0;
        if (std::fabs(p - std::round(p)) > 1e-12)
            return gopf_fail(c.ctx, GOPF_ERR_UNSUPPORTED, "non-integer power in '" + desc + "' has no device implementation");
        dv.nfac++;
    }
    c.d.derived.push_back(dv);
    c.d.derived_names.push_back(desc);
    return GOPF_OK;
}

// pf/model.go:165-195
int update_derived_fields(Ctx &c, const std::string &eq)
{
    std::vector<std::string> sides = split(eq, '=');
    if (sides.size() != 2) return parse_fail(c.ctx, "equality sign can only occur once");
    std::string field;
    if (!field_from_leibniz(sides[0], field)) return parse_fail(c.ctx, "'" + sides[0] + "' is not a Leibniz derivative");
    for (auto &sd : split_on_many(sides[1], {"+", "-"})) {
        int kind;
        if (c.user_term(sd.sub, kind) >= 0) continue;
        std::string nf = sort_factors(non_linear_field_expressions(sd.sub, field, c.d.fields));
        if (!nf.empty() && !c.is_field_name(nf)) {
            int rc = add_product_derived(c, nf);
            if (rc) return rc;
        }
    }
    return GOPF_OK;
}

// ConcreteTerm (pf/rhsBuilder.go:125-190) -> coef, lap, source
int concrete_term(Ctx &c, const SubDelim &t, int eq, int implicit, std::vector<gopf_term> &out)
{
    const std::string &term = t.sub;
    const double sign = (t.delim == "-") ? -1.0 : 1.0;
    std::complex<double> coef(sign, 0.0);
    for (auto &r : star_runs(term)) {
        std::string name = r.substr(0, r.find('^'));
        if (!c.is_field_name(name) && c.is_brick(name)) {
            double p;
            if (!get_power(r, p)) return parse_fail(c.ctx, "bad power in '" + r + "'");
            coef *= std::pow(c.d.scalars.at(name), std::complex<double>(p, 0.0));
        } else if (!c.valid_name(name)) {
            return parse_fail(c.ctx, "Name " + name + " is not defined!");
        }
    }
    if (std::fabs(coef.imag()) > 1e-12 * std::max(1.0, std::fabs(coef.real())))
        return gopf_fail(c.ctx, GOPF_ERR_UNSUPPORTED, "complex-valued coefficient in '" + term + "'");
    std::string fname = get_field_name(sort_factors(term), c.all_field_names());
    int lap = 0;
    if (contains(term, "LAP")) {
        static const std::regex rl("LAP*[^a-zA-Z]*");
        std::smatch m;
        std::string res;
        if (std::regex_search(term, m, rl)) res = m[0].str();
        double p;
        if (!get_power(res, p)) return parse_fail(c.ctx, "bad LAP power in '" + term + "'");
        lap = (int)p;
    }
    gopf_term gt;
    memset(&gt, 0, sizeof(gt));
    gt.eq = eq;
    gt.implicit = implicit;
    gt.coef = coef.real();
    gt.lap = lap;
    if (fname.empty()) {
        gt.source = GOPF_SRC_NONE;
    } else {
        int fid = -1;
        for (size_t i = 0; i < c.d.fields.size(); ++i)
            if (c.d.fields[i] == fname) fid = (int)i;
        if (fid >= 0) {
            gt.source = GOPF_SRC_FIELD;
            gt.src_index = fid;
        } else {
            int did = -1;
            for (size_t i = 0; i < c.d.derived_names.size(); ++i)
                if (c.d.derived_names[i] == fname) did = (int)i;
            if (did < 0) return parse_fail(c.ctx, "unknown brick '" + fname + "'");
            gt.source = GOPF_SRC_DERIVED;
            gt.src_index = did;
        }
    }
    out.push_back(gt);
    return GOPF_OK;
}

// pf.Build (pf/rhsBuilder.go:26-54)
int build(Ctx &c, const std::string &eq, int eqidx, std::vector<gopf_term> &terms, std::vector<gopf_special> &specials)
{
    std::vector<std::string> sides = split(eq, '=');
    if (sides.size() != 2) return parse_fail(c.ctx, "build: equality sign can only occur once");
    std::string field;
    if (!field_from_leibniz(sides[0], field))
        return parse_fail(c.ctx, "rhsbuilder: Passed string is not a leibniz formatted string");
    for (auto &t : split_on_many(sides[1], {"+", "-"})) {
        std::string name = remove_known_prefixes(t.sub);
        std::vector<std::string> prefixes = get_known_prefixes(t.sub);
        prefixes.push_back(t.delim);
        int kind = 0;
        int ut = c.user_term(name, kind);
        if (ut >= 0) {
            double s = 1.0;
            int lap = 0;
            for (auto &p : prefixes) {
                if (p == "-") s = -s;
                else if (p == "LAP^4") lap += 4;
                else if (p == "LAP^2") lap += 2;
                else if (p == "LAP") lap += 1;
            }
            specials.push_back({kind, ut, eqidx, s, lap});
            continue;
        }
        if (is_bilinear(t.sub, field, c.all_field_names())) {
            SubDelim tt = t;
            tt.sub = replace_all(tt.sub, field, "");
            int rc = concrete_term(c, tt, eqidx, 1, terms);
            if (rc) return rc;
        } else {
            int rc = concrete_term(c, t, eqidx, 0, terms);
            if (rc) return rc;
        }
    }
    return GOPF_OK;
}

} // namespace

static bool name_is_reserved(const std::string &name) { return !get_known_prefixes(name).empty(); }

extern "C" int gopf_add_field(gopf_ctx *ctx, const char *name, int *field_id)
{
    if (!ctx || !name || !*name) return gopf_fail(ctx, GOPF_ERR_ARG, "field name required");
    if (name_is_reserved(name))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    for (auto &f : ctx->def.fields)
        if (f == name) return gopf_fail(ctx, GOPF_ERR_ARG, std::string("field '") + name + "' already exists");
    ctx->def.fields.push_back(name);
    if (field_id) *field_id = (int)ctx->def.fields.size() - 1;
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_add_scalar(gopf_ctx *ctx, const char *name, double re, double im)
{
    if (!ctx || !name || !*name) return gopf_fail(ctx, GOPF_ERR_ARG, "scalar name required");
    if (name_is_reserved(name))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    ctx->def.scalars[name] = std::complex<double>(re, im);
    ctx->initialised = false;
    return GOPF_OK;
}

static int field_index(gopf_ctx *ctx, const char *field)
{
    if (!field) return -1;
    for (size_t i = 0; i < ctx->def.fields.size(); ++i)
        if (ctx->def.fields[i] == field) return (int)i;
    return -1;
}

extern "C" int gopf_register_function(gopf_ctx *ctx, const char *name, int kind, const char *field, const double *coefs,
                                      const int *powers, int nterms)
{
    if (!ctx || !name || !*name) return gopf_fail(ctx, GOPF_ERR_ARG, "function name required");
    if (name_is_reserved(name))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    int fid = field_index(ctx, field);
    if (fid < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown field");
    gopf_derived dv;
    memset(&dv, 0, sizeof(dv));
    dv.kind = kind;
    if (kind == GOPF_DER_POLY) {
        if (nterms < 1 || nterms > GOPF_MAX_FACTORS || !coefs || !powers)
            return gopf_fail(ctx, GOPF_ERR_ARG, "polynomial needs 1..8 terms");
        dv.nfac = nterms;
        for (int i = 0; i < nterms; ++i) {
            dv.field[i] = fid;
            dv.power[i] = powers[i];
            dv.coef[i] = coefs[i];
        }
    } else if (kind == GOPF_DER_INDICATOR || kind == GOPF_DER_INDICATOR_D || kind == GOPF_DER_INDICATOR_HD) {
        dv.nfac = 1;
        dv.field[0] = fid;
        dv.power[0] = 1;
        dv.coef[0] = 1.0;
    } else {
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "function kind has no device implementation");
    }
    ctx->def.derived.push_back(dv);
    ctx->def.derived_names.push_back(name);
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_register_polynomial(gopf_ctx *ctx, const char *name, const double *coefs, const int *powers,
                                        int nterms, int nfields)
{
    if (!ctx || !name || !*name) return gopf_fail(ctx, GOPF_ERR_ARG, "function name required");
    if (name_is_reserved(name))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    if (nterms < 1 || nterms > GOPF_MAX_FACTORS || !coefs || !powers)
        return gopf_fail(ctx, GOPF_ERR_ARG, "polynomial needs 1..8 terms");
    if (nfields < 1 || nfields > 4 || nfields > (int)ctx->def.fields.size())
        return gopf_fail(ctx, GOPF_ERR_ARG, "powers must cover 1..4 fields that have been added");
    gopf_derived dv;
    memset(&dv, 0, sizeof(dv));
    dv.kind = GOPF_DER_MPOLY;
    dv.nfac = nterms;
    for (int t = 0; t < nterms; ++t) {
        unsigned packed = 0;
        for (int f = 0; f < nfields; ++f) {
            const int p = powers[t * nfields + f];
            if (p < 0 || p > 64) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "powers are 0..64 on the device");
            packed |= (unsigned)p << (8 * f);
        }
        dv.power[t] = (int)packed;
        dv.coef[t] = coefs[t];
        dv.field[t] = -1;
    }
    ctx->def.derived.push_back(dv);
    ctx->def.derived_names.push_back(name);
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_register_elastic(gopf_ctx *ctx, const char *term, const char *field, const double *C81,
                                     const double *misfit9)
{
    if (!ctx || !term || !*term || !C81 || !misfit9) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    int fid = field_index(ctx, field);
    if (fid < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown field");
    gopf_modeldef::Elastic e;
    e.name = term;
    e.field = fid;
    memcpy(e.C, C81, sizeof(e.C));
    memcpy(e.misfit, misfit9, sizeof(e.misfit));
    ctx->def.elastic.push_back(e);
    ctx->initialised = false;
    return GOPF_OK;
}

// RegisterImplicitTerm(name, &TensorialHessian{K: K}, nil) (pf/tensorialHessian.go:38-80)
extern "C" int gopf_register_hessian(gopf_ctx *ctx, const char *term, const double *K, int nk)
{
    if (!ctx || !term || !*term || !K) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    if (name_is_reserved(term))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    if (nk != 4 && nk != 9) return gopf_fail(ctx, GOPF_ERR_ARG, "K has 4 (2D) or 9 (3D) entries");
    gopf_modeldef::ImplicitSym h{};
    h.name = term;
    h.kind = 1;
    h.nk = nk;
    memcpy(h.K, K, sizeof(double) * (size_t)nk);
    ctx->def.isym.push_back(h);
    ctx->initialised = false;
    return GOPF_OK;
}

// RegisterImplicitTerm(name, &SpectralViscosity{Eps, DissipationThreshold, Power}, nil)
// (pf/spectralViscosity.go:22-58)
extern "C" int gopf_register_spectral_viscosity(gopf_ctx *ctx, const char *term, double eps, double threshold,
                                                int power)
{
    if (!ctx || !term || !*term) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    if (name_is_reserved(term))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    if (!(threshold > 0.0) || power < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "threshold > 0 and power >= 0 required");
    gopf_modeldef::ImplicitSym v{};
    v.name = term;
    v.kind = 2;
    v.eps = eps;
    v.threshold = threshold;
    v.power = power;
    ctx->def.isym.push_back(v);
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_register_volcons(gopf_ctx *ctx, const char *term, const char *field, const char *indicator, double dt)
{
    if (!ctx || !term || !*term || !indicator) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    int fid = field_index(ctx, field);
    if (fid < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown field");
    gopf_modeldef::Volcons v;
    v.name = term;
    v.field = fid;
    v.indicator = indicator;
    v.dt = dt;
    ctx->def.volcons.push_back(v);
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_register_noise(gopf_ctx *ctx, const char *name, int kind, const char *field, double strength,
                                   unsigned long long seed)
{
    if (!ctx || !name || !*name) return gopf_fail(ctx, GOPF_ERR_ARG, "noise name required");
    if (name_is_reserved(name))
        return gopf_fail(ctx, GOPF_ERR_ARG, "names may not start with the reserved words -, LAP^4, LAP^2, LAP, *");
    if (kind != GOPF_NOISE_WHITE && kind != GOPF_NOISE_CONSERVATIVE) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown noise kind");
    if (!(strength >= 0.0)) return gopf_fail(ctx, GOPF_ERR_ARG, "noise strength must be >= 0");
    int fid = field_index(ctx, field);
    if (fid < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown field");
    ctx->def.noise.push_back({name, kind, fid, strength, seed});
    if (kind == GOPF_NOISE_WHITE) { // a derived field brick, as RegisterFunction does
        gopf_derived dv;
        memset(&dv, 0, sizeof(dv));
        dv.kind = GOPF_DER_WHITE_NOISE;
        dv.nfac = 1;
        dv.field[0] = fid;
        dv.coef[0] = strength;
        ctx->def.derived.push_back(dv);
        ctx->def.derived_names.push_back(name);
    }
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_add_equation(gopf_ctx *ctx, const char *equation)
{
    if (!ctx || !equation) return gopf_fail(ctx, GOPF_ERR_ARG, "null equation");
    std::string eq = replace_all(equation, " ", "");
    Ctx c{ctx, ctx->def};
    int rc = update_derived_fields(c, eq);
    if (rc) return rc;
    ctx->def.equations.push_back(eq);
    ctx->initialised = false;
    return GOPF_OK;
}

extern "C" int gopf_init(gopf_ctx *ctx)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (ctx->def.fields.empty()) return gopf_fail(ctx, GOPF_ERR_STATE, "Model: No fields added");
    if (ctx->def.equations.size() != ctx->def.fields.size())
        return gopf_fail(ctx, GOPF_ERR_STATE, "one equation per field is required (equation i evolves field i)");
    Ctx c{ctx, ctx->def};
    std::vector<gopf_term> terms;
    std::vector<gopf_special> specials;
    for (size_t i = 0; i < ctx->def.equations.size(); ++i) {
        std::string field;
        field_from_leibniz(split(ctx->def.equations[i], '=')[0], field);
        if (field != ctx->def.fields[i])
            return gopf_fail(ctx, GOPF_ERR_STATE, "equation " + std::to_string(i) + " evolves '" + field +
                                                      "' but field " + std::to_string(i) + " is '" +
                                                      ctx->def.fields[i] + "'");
        int rc = build(c, ctx->def.equations[i], (int)i, terms, specials);
        if (rc) return rc;
    }
    if (ctx->device >= 0) {
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, cudaGetErrorString(e));
    }
    ctx->nfields = (int)ctx->def.fields.size();
    ctx->der = ctx->def.derived;
    ctx->terms = terms;
    ctx->specials = specials;
    return gopf_compile_model(ctx);
}
