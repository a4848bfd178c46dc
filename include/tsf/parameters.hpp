// parameters.hpp -- the parameter system of the Tube Segmentation Framework
// API (reference parameters.hpp:20-91): typed parameters with range /
// possibility validation, the schema file `parameters`, presets under
// centerline-{gpu,ridge,test}/<name>, and command-line parsing.  Same class
// and function names, argument meaning and exceptions as the reference.
#ifndef TSF_PARAMETERS_HPP
#define TSF_PARAMETERS_HPP

#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

using std::unordered_map;

class BoolParameter {
public:
    BoolParameter() {}
    BoolParameter(bool defaultValue, std::string description, std::string group);
    bool get();
    void set(bool value);
    std::string getDescription() const;
    std::string getGroup() const;
    void setGroup(std::string group);

private:
    bool value = false;
    std::string description;
    std::string group;
};

class NumericParameter {
public:
    NumericParameter() {}
    NumericParameter(float defaultValue, float min, float max, float step, std::string description,
                     std::string group);
    float get();
    void set(float value);            // throws SIPL::SIPLException outside [min, max]
    bool validate(float value);
    float getMax() const;
    void setMax(float max);
    float getMin() const;
    void setMin(float min);
    float getStep() const;
    void setStep(float step);
    std::string getDescription() const;
    std::string getGroup() const;
    void setGroup(std::string group);

private:
    float value = 0.0f;
    float min = 0.0f;
    float max = 0.0f;
    float step = 0.0f;
    std::string description;
    std::string group;
};

class StringParameter {
public:
    StringParameter() {}
    StringParameter(std::string defaultValue, std::vector<std::string> possibilities, std::string description,
                    std::string group);
    std::string get();
    void set(std::string value);      // throws SIPL::SIPLException if not one of the possibilities
    void setWithoutValidation(std::string value);
    bool validate(std::string value);
    std::vector<std::string> getPossibilities() const;
    std::string getDescription() const;
    std::string getGroup() const;
    void setGroup(std::string group);

private:
    std::string value;
    std::vector<std::string> possibilities;
    std::string description;
    std::string group;
};

typedef struct paramList {
    unordered_map<std::string, BoolParameter> bools;
    unordered_map<std::string, NumericParameter> numerics;
    unordered_map<std::string, StringParameter> strings;
} paramList;

// parameters.cpp:67-106 -- apply parameter_dir/centerline-<method>/<preset>
void loadParameterPreset(paramList &parameters, std::string parameter_dir);
// parameters.cpp:108-172 -- read parameter_dir/parameters (throws SIPL::IOException)
paramList initParameters(std::string parameter_dir);
// parameters.cpp:174-200 -- set by name (throws SIPL::SIPLException)
void setParameter(paramList &parameters, std::string name, std::string value);
// parameters.cpp:227-270 -- argv[1] is the file name, then --name [value] ...
paramList getParameters(int argc, char **argv);
float getParam(paramList parameters, std::string parameterName);
bool getParamBool(paramList parameters, std::string parameterName);
std::string getParamStr(paramList parameters, std::string parameterName);
void printAllParameters();

// Directory holding the `parameters` schema and the preset folders shipped
// with the library (the reference's compile-time PARAMETERS_DIR).  The
// environment variable TSF_PARAMETERS_DIR overrides it.
const char *tsf_parameters_dir();

#ifndef PARAMETERS_DIR
#define PARAMETERS_DIR tsf_parameters_dir()
#endif
#ifndef KERNELS_DIR
#define KERNELS_DIR ""
#endif

#endif
