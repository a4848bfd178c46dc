// parameters.cpp -- the parameter system (interface of reference
// parameters.hpp / parameters.cpp; the schema file format is the reference's:
// `name type default [min max step | possibilities...] "description" group`).
#include "tsf/parameters.hpp"

#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <locale>
#include <sstream>

#include "tsf/SIPL/Exceptions.hpp"

namespace {

float parse_float(const std::string &s) {
    std::istringstream in(s);
    in.imbue(std::locale::classic());
    float v = 0.0f;
    in >> v;
    return v;
}

// Splits a schema line into whitespace-separated tokens, keeping the quoted
// description as one token (without its quotes).  Returns false for blank or
// comment lines.
bool tokenize(const std::string &line, std::vector<std::string> &tok, std::string &description, std::string &group) {
    tok.clear();
    description.clear();
    group.clear();
    const size_t q0 = line.find('"');
    if (line.empty() || line[0] == '#' || q0 == std::string::npos) return false;
    const size_t q1 = line.find('"', q0 + 1);
    if (q1 == std::string::npos) return false;
    std::istringstream head(line.substr(0, q0));
    std::string t;
    while (head >> t) tok.push_back(t);
    description = line.substr(q0 + 1, q1 - q0 - 1);
    std::istringstream tail(line.substr(q1 + 1));
    tail >> group;
    return tok.size() >= 3;
}

std::string strip(const std::string &s) {
    size_t b = 0, e = s.size();
    while (b < e && (s[b] == ' ' || s[b] == '\t' || s[b] == '\r' || s[b] == '\n')) b++;
    while (e > b && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r' || s[e - 1] == '\n')) e--;
    return s.substr(b, e - b);
}

}  // namespace

// ---- BoolParameter ---------------------------------------------------------
BoolParameter::BoolParameter(bool defaultValue, std::string description_, std::string group_)
    : value(defaultValue), description(description_), group(group_) {}
bool BoolParameter::get() { return value; }
void BoolParameter::set(bool v) { value = v; }
std::string BoolParameter::getDescription() const { return description; }
std::string BoolParameter::getGroup() const { return group; }
void BoolParameter::setGroup(std::string g) { group = g; }

// ---- NumericParameter --------------------------------------------------------
NumericParameter::NumericParameter(float defaultValue, float min_, float max_, float step_, std::string description_,
                                   std::string group_)
    : min(min_), max(max_), step(step_), description(description_), group(group_) {
    set(defaultValue);
}
float NumericParameter::get() { return value; }
void NumericParameter::set(float v) {
    if (!validate(v)) throw SIPL::SIPLException("Error in setting numerical parameter ", __LINE__, __FILE__);
    value = v;
}
bool NumericParameter::validate(float v) { return v >= min && v <= max; }
float NumericParameter::getMax() const { return max; }
void NumericParameter::setMax(float m) { max = m; }
float NumericParameter::getMin() const { return min; }
void NumericParameter::setMin(float m) { min = m; }
float NumericParameter::getStep() const { return step; }
void NumericParameter::setStep(float s) { step = s; }
std::string NumericParameter::getDescription() const { return description; }
std::string NumericParameter::getGroup() const { return group; }
void NumericParameter::setGroup(std::string g) { group = g; }

// ---- StringParameter -----------------------------------------------------------
StringParameter::StringParameter(std::string defaultValue, std::vector<std::string> possibilities_,
                                 std::string description_, std::string group_)
    : possibilities(possibilities_), description(description_), group(group_) {
    set(defaultValue);
}
std::string StringParameter::get() { return value; }
void StringParameter::set(std::string v) {
    if (!validate(v)) throw SIPL::SIPLException("Error in setting string parameter", __LINE__, __FILE__);
    value = v;
}
void StringParameter::setWithoutValidation(std::string v) { value = v; }
bool StringParameter::validate(std::string v) {
    if (possibilities.empty()) return true;
    for (const auto &p : possibilities)
        if (p == v) return true;
    return false;
}
std::vector<std::string> StringParameter::getPossibilities() const { return possibilities; }
std::string StringParameter::getDescription() const { return description; }
std::string StringParameter::getGroup() const { return group; }
void StringParameter::setGroup(std::string g) { group = g; }

// ---- schema, presets, lookup -------------------------------------------------------
paramList initParameters(std::string parameter_dir) {
    const std::string filename = parameter_dir + "/parameters";
    std::ifstream file(filename.c_str());
    if (!file.is_open()) throw SIPL::IOException(filename.c_str(), __LINE__, __FILE__);
    paramList parameters;
    std::string line, description, group;
    std::vector<std::string> tok;
    while (std::getline(file, line)) {
        if (!tokenize(line, tok, description, group)) continue;
        const std::string &name = tok[0], &type = tok[1], &def = tok[2];
        if (type == "bool") {
            parameters.bools[name] = BoolParameter(def == "true", description, group);
        } else if (type == "num") {
            if (tok.size() < 6) throw SIPL::SIPLException(("Could not parse parameter " + name).c_str());
            parameters.numerics[name] = NumericParameter(parse_float(def), parse_float(tok[3]), parse_float(tok[4]),
                                                         parse_float(tok[5]), description, group);
        } else if (type == "str") {
            std::vector<std::string> poss(tok.begin() + 3, tok.end());
            parameters.strings[name] = StringParameter(def, poss, description, group);
        } else {
            const std::string msg = "Could not parse parameter of type: " + type;
            throw SIPL::SIPLException(msg.c_str());
        }
    }
    return parameters;
}

void setParameter(paramList &parameters, std::string name, std::string value) {
    if (parameters.bools.count(name) > 0) {
        parameters.bools[name].set(value == "true");
    } else if (parameters.numerics.count(name) > 0) {
        parameters.numerics[name].set(parse_float(value));
    } else if (parameters.strings.count(name) > 0) {
        if (name == "parameters") parameters.strings[name].setWithoutValidation(value);
        else parameters.strings[name].set(value);
    } else {
        const std::string msg = "Can not set value for parameter with name: " + name;
        throw SIPL::SIPLException(msg.c_str());
    }
}

void loadParameterPreset(paramList &parameters, std::string parameter_dir) {
    const std::string preset = getParamStr(parameters, "parameters");
    if (preset == "none") return;
    const std::string method = getParamStr(parameters, "centerline-method");
    if (method != "gpu" && method != "test" && method != "ridge") return;
    const std::string filename = parameter_dir + "/centerline-" + method + "/" + preset;
    std::ifstream file(filename.c_str());
    if (!file.is_open()) throw SIPL::IOException(filename.c_str());
    std::string line;
    while (std::getline(file, line)) {
        line = strip(line);
        if (line.empty()) continue;
        const size_t sp = line.find(' ');
        if (sp != std::string::npos) setParameter(parameters, line.substr(0, sp), strip(line.substr(sp + 1)));
        else setParameter(parameters, line, "true");
    }
}

float getParam(paramList parameters, std::string name) {
    if (parameters.numerics.count(name) == 0)
        throw SIPL::SIPLException(("numeric parameter not found: " + name).c_str());
    return parameters.numerics[name].get();
}

bool getParamBool(paramList parameters, std::string name) {
    if (parameters.bools.count(name) == 0) throw SIPL::SIPLException(("bool parameter not found: " + name).c_str());
    return parameters.bools[name].get();
}

std::string getParamStr(paramList parameters, std::string name) {
    if (parameters.strings.count(name) == 0)
        throw SIPL::SIPLException(("string parameter not found: " + name).c_str());
    return parameters.strings[name].get();
}

paramList getParameters(int argc, char **argv) {
    paramList parameters = initParameters(PARAMETERS_DIR);
    // first pass: the preset and the centerline method decide which preset file applies
    for (int i = 2; i < argc; i++) {
        const std::string token = argv[i];
        if (token.substr(0, 2) != "--") continue;
        std::string next;
        if (i + 1 < argc) {
            next = argv[i + 1];
            if (next.substr(0, 2) != "--") i++;
            else next.clear();
        }
        const std::string name = token.substr(2);
        if (name == "parameters" || name == "centerline-method") setParameter(parameters, name, next);
    }
    loadParameterPreset(parameters, PARAMETERS_DIR);
    // second pass: every --name [value]; a flag without value means "true"
    for (int i = 2; i < argc; i++) {
        const std::string token = argv[i];
        if (token.substr(0, 2) != "--") continue;
        std::string next = "true";
        if (i + 1 < argc) {
            const std::string cand = argv[i + 1];
            if (cand.substr(0, 2) != "--") {
                next = cand;
                i++;
            }
        }
        setParameter(parameters, token.substr(2), next);
    }
    return parameters;
}

void printAllParameters() {
    paramList parameters = initParameters(PARAMETERS_DIR);
    std::printf("%25s \t Default \t Range \t\t\t Description\n", "Name");
    std::cout << std::string(102, '-') << std::endl;
    for (auto &b : parameters.bools)
        std::printf("%25s \t %s \t\t true/false \t\t %s \n", b.first.c_str(), b.second.get() ? "true" : "false",
                    b.second.getDescription().c_str());
    for (auto &n : parameters.numerics) {
        if (n.second.getStep() >= 1.0f)
            std::printf("%25s \t %.0f \t\t %.0f-%.0f \t\t %s \n", n.first.c_str(), n.second.get(), n.second.getMin(),
                        n.second.getMax(), n.second.getDescription().c_str());
        else
            std::printf("%25s \t %.3f \t\t %.3f-%.3f \t\t %s \n", n.first.c_str(), n.second.get(), n.second.getMin(),
                        n.second.getMax(), n.second.getDescription().c_str());
    }
    for (auto &s : parameters.strings) {
        std::string poss;
        for (const auto &p : s.second.getPossibilities()) poss += p + " ";
        std::printf("%25s \t %s \t\t %s \t\t %s\n", s.first.c_str(), s.second.get().c_str(), poss.c_str(),
                    s.second.getDescription().c_str());
    }
}

// The schema and presets ship in <package>/parameters; the library sits in
// <package>/lib.
const char *tsf_parameters_dir() {
    static std::string dir;
    if (dir.empty()) {
        const char *env = std::getenv("TSF_PARAMETERS_DIR");
        if (env && *env) {
            dir = env;
        } else {
            Dl_info info;
            if (dladdr((void *)&tsf_parameters_dir, &info) && info.dli_fname) {
                std::string p = info.dli_fname;
                const size_t s1 = p.rfind('/');
                p = (s1 == std::string::npos) ? "." : p.substr(0, s1);     // .../lib
                const size_t s2 = p.rfind('/');
                p = (s2 == std::string::npos) ? "." : p.substr(0, s2);     // package dir
                dir = p + "/parameters";
            } else {
                dir = "parameters";
            }
        }
    }
    return dir.c_str();
}
