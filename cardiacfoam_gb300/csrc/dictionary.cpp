// Reader for the subset of OpenFOAM dictionary syntax used by
// constant/electroProperties, and cfg_monodomain_create_from_dict, which
// applies the reference's keys and selection rules:
//   myocardiumSolver <name>;  <name>Coeffs { ... }      (electroModel.C:142-200)
//   conductivity [dims] (xx xy xz yy yz zz);            (monodomainSolver.C:86-95)
//   chi / cm [dims] value;                              (myocardiumDomain.C:265-266)
//   ionicModel, tissue, solver, absTol, relTol, maxSteps (ionicModel.C:76-94)
//   solutionAlgorithm implicit|explicit                 (myocardiumDomain.C:271-277)
//   explicit: deltaT = maxCo min(dx^2/Df)                (electroModel.C:238-257)
//   externalStimulus { ... }                            (stimulusIO.C:305-400)
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "host_common.h"

namespace cfg {
namespace {

struct Entry;
using Dict = std::map<std::string, std::shared_ptr<Entry>>;

struct Entry {
    bool is_dict = false;
    std::vector<std::string> tokens;   // value tokens, "(" ")" kept, [dims] dropped
    Dict dict;
    std::vector<std::string> order;    // keys of dict in the order they first appear
};

class Parser {
public:
    explicit Parser(const std::string& s) : s_(s) {}

    bool parse(Dict& out, std::string& err)
    {
        try {
            parse_body(out, false);
        } catch (const std::string& e) {
            err = e;
            return false;
        }
        return true;
    }

private:
    const std::string& s_;
    size_t i_ = 0;

    void skip()
    {
        for (;;) {
            while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
            if (s_.compare(i_, 2, "//") == 0) {
                while (i_ < s_.size() && s_[i_] != '\n') ++i_;
            } else if (s_.compare(i_, 2, "/*") == 0) {
                size_t e = s_.find("*/", i_ + 2);
                i_ = e == std::string::npos ? s_.size() : e + 2;
            } else {
                return;
            }
        }
    }

    std::string token()
    {
        skip();
        if (i_ >= s_.size()) return "";
        const char c = s_[i_];
        if (std::strchr("(){}[];", c)) {
            ++i_;
            return std::string(1, c);
        }
        if (c == '"') {
            size_t e = s_.find('"', i_ + 1);
            if (e == std::string::npos) throw std::string("unterminated string");
            std::string t = s_.substr(i_ + 1, e - i_ - 1);
            i_ = e + 1;
            return t;
        }
        size_t b = i_;
        while (i_ < s_.size() && !std::isspace((unsigned char)s_[i_]) &&
               !std::strchr("(){}[];", s_[i_]))
            ++i_;
        return s_.substr(b, i_ - b);
    }

    std::string peek()
    {
        size_t save = i_;
        std::string t = token();
        i_ = save;
        return t;
    }

    void parse_body(Dict& d, bool nested, std::vector<std::string>* order = nullptr)
    {
        for (;;) {
            std::string key = token();
            if (key.empty()) {
                if (nested) throw std::string("missing '}'");
                return;
            }
            if (key == "}") {
                if (!nested) throw std::string("unexpected '}'");
                return;
            }
            if (key == ";") continue;
            if (key[0] == '#') {   // directives (#include, #inputMode) are not followed
                while (!token().empty() && peek() != ";" && s_[i_ - 1] != '\n') {}
                continue;
            }
            auto e = std::make_shared<Entry>();
            if (peek() == "{") {
                token();
                e->is_dict = true;
                parse_body(e->dict, true, &e->order);
            } else {
                int depth = 0;
                for (;;) {
                    std::string t = token();
                    if (t.empty()) throw std::string("missing ';' after " + key);
                    if (t == "[") {   // dimension set: dropped
                        while (true) {
                            std::string u = token();
                            if (u.empty()) throw std::string("missing ']'");
                            if (u == "]") break;
                        }
                        continue;
                    }
                    if (t == "(") ++depth;
                    if (t == ")") --depth;
                    if (t == ";" && depth == 0) break;
                    e->tokens.push_back(t);
                }
            }
            if (order && d.find(key) == d.end()) order->push_back(key);
            d[key] = e;
        }
    }
};

const Entry* find(const Dict& d, const char* k)
{
    auto it = d.find(k);
    return it == d.end() ? nullptr : it->second.get();
}

bool scalar(const Dict& d, const char* k, double& v)
{
    const Entry* e = find(d, k);
    if (!e || e->is_dict || e->tokens.empty()) return false;
    // "name value" (dimensionedScalar with a name) or "value"
    const std::string& t = e->tokens.back();
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == '\0';
}

bool word(const Dict& d, const char* k, std::string& v)
{
    const Entry* e = find(d, k);
    if (!e || e->is_dict || e->tokens.empty()) return false;
    v = e->tokens[0];
    return true;
}

// numbers inside the (possibly nested) list of an entry
std::vector<double> numbers(const Entry* e)
{
    std::vector<double> out;
    if (!e) return out;
    for (const std::string& t : e->tokens) {
        if (t == "(" || t == ")") continue;
        char* end = nullptr;
        double v = std::strtod(t.c_str(), &end);
        if (end && *end == '\0') out.push_back(v);
    }
    return out;
}

// ionicModel, tissue and the ODE solver keys of <type>Coeffs
// (ionicModel.C:76-94); the strings live in thread-local storage until the
// next call on the thread.
int parse_ionic(const Dict& c, long long n_cells, double delta_t, int precision,
                cfg_ionic_desc& io)
{
    static thread_local std::string model, tissue, ode_solver;
    if (!word(c, "ionicModel", model))
        return fail(CFG_ERR_INVALID, "keyword ionicModel is undefined");
    if (!word(c, "tissue", tissue)) tissue.clear();
    io.ionic_model = model.c_str();
    io.tissue = tissue.empty() ? nullptr : tissue.c_str();
    io.n_cells = n_cells;
    io.initial_delta_t = delta_t;   // runTime.deltaT (myocardiumDomainInterface.C:71-76)
    io.solve_vm_within_ode = 0;
    io.precision = precision;
    io.ode.solver = word(c, "solver", ode_solver) ? ode_solver.c_str() : "RKF45";
    double v;
    io.ode.abs_tol = scalar(c, "absTol", v) ? v : -1;
    io.ode.rel_tol = scalar(c, "relTol", v) ? v : -1;
    io.ode.max_steps = scalar(c, "maxSteps", v) ? (long long)v : -1;
    io.ode.safe_scale = scalar(c, "safeScale", v) ? v : -1;
    io.ode.min_scale = scalar(c, "minScale", v) ? v : -1;
    io.ode.max_scale = scalar(c, "maxScale", v) ? v : -1;
    io.ode.alpha_increase = scalar(c, "alphaIncrease", v) ? v : -1;
    io.ode.alpha_decrease = scalar(c, "alphaDecrease", v) ? v : -1;
    return CFG_OK;
}

// externalStimulus (stimulusIO::loadExternalStimulusProtocol) into the box
// fields of a monodomain or bidomain description
template <class D>
int parse_stimulus(const Dict& c, D& d)
{
    if (const Entry* se = find(c, "externalStimulus"); se && se->is_dict) {
        const Dict& s = se->dict;
        std::vector<double> mn, mx;
        const bool lists = find(s, "stimulusLocationMinList") != nullptr;
        if (lists != (find(s, "stimulusLocationMaxList") != nullptr))
            return fail(CFG_ERR_INVALID, "Both stimulusLocationMinList and "
                                         "stimulusLocationMaxList must be provided together.");
        mn = numbers(find(s, lists ? "stimulusLocationMinList" : "stimulusLocationMin"));
        mx = numbers(find(s, lists ? "stimulusLocationMaxList" : "stimulusLocationMax"));
        if (mn.size() != mx.size() || mn.empty() || mn.size() % 3)
            return fail(CFG_ERR_INVALID, "stimulus box corners are inconsistent");
        const int nb = int(mn.size() / 3);
        if (nb > 8) return fail(CFG_ERR_UNSUPPORTED, "at most 8 stimulus boxes");
        d.n_boxes = nb;
        auto per_box = [&](const char* list, const char* single, double* dst, bool required,
                           double dflt) -> int {
            std::vector<double> l = numbers(find(s, list));
            if (!l.empty()) {
                if (int(l.size()) != nb)
                    return fail(CFG_ERR_INVALID, "%s has %d entries, expected %d", list,
                                int(l.size()), nb);
                for (int b = 0; b < nb; ++b) dst[b] = l[size_t(b)];
                return CFG_OK;
            }
            double x = dflt;
            if (!scalar(s, single, x) && required)
                return fail(CFG_ERR_INVALID, "keyword %s is undefined", single);
            for (int b = 0; b < nb; ++b) dst[b] = x;
            return CFG_OK;
        };
        int rc;
        if ((rc = per_box("stimulusStartTimeList", "stimulusStartTime", d.box_start, false, 0.0)))
            return rc;
        if ((rc = per_box("stimulusDurationList", "stimulusDuration", d.box_duration, true, 0.0)))
            return rc;
        if ((rc = per_box("stimulusIntensityList", "stimulusIntensity", d.box_intensity, true,
                          0.0)))
            return rc;
        for (int b = 0; b < nb; ++b) {
            if (d.box_duration[b] < 0)
                return fail(CFG_ERR_INVALID, "stimulusDuration must be non-negative");
            for (int k = 0; k < 3; ++k) {
                d.box_min[b][k] = mn[size_t(3 * b + k)];
                d.box_max[b][k] = mx[size_t(3 * b + k)];
            }
        }
    }
    return CFG_OK;
}

}  // namespace
}  // namespace cfg

using namespace cfg;

extern "C" int cfg_monodomain_create_from_dict(const char* text, const cfg_mesh_desc* mesh,
                                               double delta_t, int precision,
                                               cfg_monodomain** out)
{
    clear_error();
    if (!text || !mesh || !out) return fail(CFG_ERR_INVALID, "null argument");
    Dict root;
    std::string err;
    std::string src(text);
    if (!Parser(src).parse(root, err))
        return fail(CFG_ERR_INVALID, "electroProperties: %s", err.c_str());
    std::string solver;
    if (!word(root, "myocardiumSolver", solver))
        return fail(CFG_ERR_INVALID, "electroProperties: keyword myocardiumSolver is undefined");
    if (solver != "monodomainSolver")
        return fail(CFG_ERR_UNSUPPORTED,
                    "myocardiumSolver %s: the monodomain context runs monodomainSolver%s",
                    solver.c_str(),
                    solver == "bidomainSolver" ? " (bidomainSolver: cfg_bidomain_create_from_dict)"
                                               : "");
    const Entry* ce = find(root, "monodomainSolverCoeffs");
    if (!ce || !ce->is_dict)
        return fail(CFG_ERR_INVALID, "electroProperties: monodomainSolverCoeffs is undefined");
    const Dict& c = ce->dict;

    cfg_monodomain_desc d{};
    if (int rc = parse_ionic(c, mesh->n_cells, delta_t, precision, d.ionic)) return rc;
    double v;

    std::vector<double> sig = numbers(find(c, "conductivity"));
    if (sig.size() != 6)
        return fail(CFG_ERR_INVALID, "conductivity must be a symmTensor (xx xy xz yy yz zz)");
    for (int k = 0; k < 6; ++k) d.conductivity[k] = sig[size_t(k)];
    if (!scalar(c, "chi", d.chi)) return fail(CFG_ERR_INVALID, "keyword chi is undefined");
    if (!scalar(c, "cm", d.cm)) return fail(CFG_ERR_INVALID, "keyword cm is undefined");
    std::string alg = "implicit";
    word(c, "solutionAlgorithm", alg);
    if (alg != "implicit" && alg != "explicit")
        return fail(CFG_ERR_INVALID, "Unrecognised solution algorithm %s", alg.c_str());
    d.implicit = alg == "implicit";
    // fvSchemes / fvSolution of the tutorials (backward; PCG 1e-8 relTol 0;
    // PIMPLE residualControl 1e-6); a "gpu" sub-dictionary may override them
    d.ddt_backward = 1;
    d.pcg_tol = 1e-8;
    d.pcg_rel_tol = 0.0;
    d.pcg_max_iter = 1000;
    d.n_outer = 1000;
    d.outer_tol = 1e-6;
    d.vm0 = -0.084;
    if (const Entry* g = find(c, "gpu"); g && g->is_dict) {
        std::string ddt;
        if (word(g->dict, "ddtScheme", ddt)) d.ddt_backward = ddt == "backward";
        if (scalar(g->dict, "tolerance", v)) d.pcg_tol = v;
        if (scalar(g->dict, "relTol", v)) d.pcg_rel_tol = v;
        if (scalar(g->dict, "maxIter", v)) d.pcg_max_iter = int(v);
        if (scalar(g->dict, "nOuterCorrectors", v)) d.n_outer = int(v);
        if (scalar(g->dict, "residualControl", v)) d.outer_tol = v;
    }
    // controlDict's maxCo (default 0.1, electroModel.C:238-257) for the
    // explicit algorithm's time step; the gpu sub-dictionary may carry it
    double max_co = 0.1;
    if (const Entry* g = find(c, "gpu"); g && g->is_dict && scalar(g->dict, "maxCo", v))
        max_co = v;
    if (int rc = parse_stimulus(c, d)) return rc;
    if (int rc = cfg_monodomain_create(&d, mesh, out)) return rc;
    if (!d.implicit) {
        // electroModel::setDeltaT: the explicit algorithm replaces deltaT once
        // with MyocardiumDomain::suggestExplicitDeltaT(maxCo)
        double dt = 0.0;
        int rc = cfg_monodomain_suggest_explicit_delta_t(*out, max_co, &dt);
        if (!rc) rc = cfg_monodomain_set_delta_t(*out, dt);
        if (rc) {
            cfg_monodomain_destroy(*out);
            *out = nullptr;
            return rc;
        }
    }
    return CFG_OK;
}

// The same for myocardiumSolver bidomainSolver: bidomainSolverCoeffs'
// conductivityIntracellular / conductivityExtracellular (symmTensors),
// phiERefPoint (required) and phiEReferenceValue (default 0)
// (bidomainSolver.C:36-127), chi, cm, the ionic model and externalStimulus as
// for the monodomain.  Solver settings follow the bidomain tutorial's
// fvSolution and fvSchemes (relTol 0, maxIter 1000 for Vm and phiE;
// nOuterCorrectors 2 without residualControl; backward ddt; Gauss linear
// gradients) except the PCG tolerance: 1e-12 instead of the tutorial's 1e-15,
// which double precision rarely reaches within maxIter (a solve that ends at
// maxIter is an error here).  A "gpu" sub-dictionary overrides any of them.
extern "C" int cfg_bidomain_create_from_dict(const char* text, const cfg_mesh_desc* mesh,
                                             double delta_t, int precision, cfg_bidomain** out)
{
    clear_error();
    if (!text || !mesh || !out) return fail(CFG_ERR_INVALID, "null argument");
    Dict root;
    std::string err;
    std::string src(text);
    if (!Parser(src).parse(root, err))
        return fail(CFG_ERR_INVALID, "electroProperties: %s", err.c_str());
    std::string solver;
    if (!word(root, "myocardiumSolver", solver))
        return fail(CFG_ERR_INVALID, "electroProperties: keyword myocardiumSolver is undefined");
    if (solver != "bidomainSolver")
        return fail(CFG_ERR_UNSUPPORTED, "myocardiumSolver %s: the bidomain context runs "
                                         "bidomainSolver", solver.c_str());
    const Entry* ce = find(root, "bidomainSolverCoeffs");
    if (!ce || !ce->is_dict)
        return fail(CFG_ERR_INVALID, "electroProperties: bidomainSolverCoeffs is undefined");
    const Dict& c = ce->dict;
    cfg_bidomain_desc d{};
    if (int rc = parse_ionic(c, mesh->n_cells, delta_t, precision, d.ionic)) return rc;
    for (int t = 0; t < 2; ++t) {
        const char* key = t == 0 ? "conductivityIntracellular" : "conductivityExtracellular";
        std::vector<double> sig = numbers(find(c, key));
        if (sig.size() != 6)
            return fail(CFG_ERR_INVALID, "%s must be a symmTensor (xx xy xz yy yz zz)", key);
        for (int k = 0; k < 6; ++k)
            (t == 0 ? d.conductivity_i : d.conductivity_e)[k] = sig[size_t(k)];
    }
    if (!scalar(c, "chi", d.chi)) return fail(CFG_ERR_INVALID, "keyword chi is undefined");
    if (!scalar(c, "cm", d.cm)) return fail(CFG_ERR_INVALID, "keyword cm is undefined");
    std::string alg = "implicit";
    word(c, "solutionAlgorithm", alg);
    if (alg != "implicit" && alg != "explicit")
        return fail(CFG_ERR_INVALID, "Unrecognised solution algorithm %s", alg.c_str());
    d.explicit_algorithm = alg == "explicit";
    std::vector<double> rp = numbers(find(c, "phiERefPoint"));
    if (rp.size() != 3) return fail(CFG_ERR_INVALID, "keyword phiERefPoint is undefined");
    for (int k = 0; k < 3; ++k) d.ref_point[k] = rp[size_t(k)];
    double v;
    d.ref_value = scalar(c, "phiEReferenceValue", v) ? v : 0.0;
    d.ddt_backward = 1;
    d.pcg_tol = d.phie_tol = 1e-12;
    d.pcg_rel_tol = d.phie_rel_tol = 0.0;
    d.pcg_max_iter = d.phie_max_iter = 1000;
    d.n_outer = 2;
    d.outer_tol = 0.0;
    d.vm0 = -0.084;
    d.grad_scheme = CFG_GRAD_GAUSS_LINEAR;
    if (const Entry* g = find(c, "gpu"); g && g->is_dict) {
        std::string w;
        if (word(g->dict, "ddtScheme", w)) d.ddt_backward = w == "backward";
        if (word(g->dict, "gradScheme", w))
            d.grad_scheme = w == "leastSquares" ? CFG_GRAD_LEAST_SQUARES : CFG_GRAD_GAUSS_LINEAR;
        if (scalar(g->dict, "tolerance", v)) d.pcg_tol = v;
        if (scalar(g->dict, "relTol", v)) d.pcg_rel_tol = v;
        if (scalar(g->dict, "maxIter", v)) d.pcg_max_iter = int(v);
        if (scalar(g->dict, "phiETolerance", v)) d.phie_tol = v;
        if (scalar(g->dict, "phiERelTol", v)) d.phie_rel_tol = v;
        if (scalar(g->dict, "phiEMaxIter", v)) d.phie_max_iter = int(v);
        if (scalar(g->dict, "nOuterCorrectors", v)) d.n_outer = int(v);
        if (scalar(g->dict, "residualControl", v)) d.outer_tol = v;
    }
    if (int rc = parse_stimulus(c, d)) return rc;
    return cfg_bidomain_create(&d, mesh, out);
}

// ECGDomain::readElectrodes (ecgDomain.C:53-82) of the ecgDomains entry in
// <myocardiumSolver>Coeffs, with the solver selection of ECGSolver::New.
extern "C" int cfg_pseudo_ecg_electrodes_from_dict(const char* text, const char* domain,
                                                   char* names, size_t len, double* positions,
                                                   int max, int* n_electrodes)
{
    clear_error();
    if (!text || !n_electrodes) return fail(CFG_ERR_INVALID, "null argument");
    *n_electrodes = 0;
    Dict root;
    std::string err;
    std::string src(text);
    if (!Parser(src).parse(root, err))
        return fail(CFG_ERR_INVALID, "electroProperties: %s", err.c_str());
    std::string solver;
    const Dict* coeffs = &root;
    if (word(root, "myocardiumSolver", solver)) {
        const Entry* ce = find(root, (solver + "Coeffs").c_str());
        if (ce && ce->is_dict) coeffs = &ce->dict;
    }
    const Entry* ed = find(*coeffs, "ecgDomains");
    if (!ed || !ed->is_dict || ed->order.empty())
        return fail(CFG_ERR_INVALID, "electroProperties: no ecgDomains");
    const std::string want = domain ? domain : "";
    const std::string name = want.empty() ? ed->order.front() : want;
    const Entry* de = find(ed->dict, name.c_str());
    if (!de || !de->is_dict) return fail(CFG_ERR_INVALID, "ecgDomains: no domain %s", name.c_str());
    std::string ecg_solver;
    if (!word(de->dict, "ecgSolver", ecg_solver))
        return fail(CFG_ERR_INVALID, "ecgDomains.%s: keyword ecgSolver is undefined", name.c_str());
    if (ecg_solver != "pseudoECG")
        return fail(CFG_ERR_UNSUPPORTED, "ecgSolver %s is not built (pseudoECG is)",
                    ecg_solver.c_str());
    const Entry* pe = find(de->dict, "electrodePositions");
    if (!pe || !pe->is_dict) return CFG_OK;   // no electrodes: an empty list
    std::string joined;
    int k = 0;
    for (const std::string& key : pe->order) {
        std::vector<double> p = numbers(find(pe->dict, key.c_str()));
        if (p.size() != 3)
            return fail(CFG_ERR_INVALID, "electrode %s: expected (x y z)", key.c_str());
        if (k < max && positions)
            for (int i = 0; i < 3; ++i) positions[3 * k + i] = p[size_t(i)];
        if (!joined.empty()) joined += ' ';
        joined += key;
        ++k;
    }
    *n_electrodes = k;
    if (k > max) return fail(CFG_ERR_INVALID, "%d electrodes, room for %d", k, max);
    if (names) {
        if (joined.size() + 1 > len) return fail(CFG_ERR_INVALID, "electrode names exceed %zu bytes", len);
        std::memcpy(names, joined.c_str(), joined.size() + 1);
    }
    return CFG_OK;
}
