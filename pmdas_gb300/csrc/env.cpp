// env.cpp — the `.env` configuration surface of the MDAS apps.
//
// Same file format and rules as the reference's Environment class
// (SDK/sutil/Environment.cpp:9-81 filterValue, :143-195 get*Value,
// :593-790 readEnvFile):
//   * `Block { key value ... }`, '#' starts a comment, words split on whitespace;
//   * an option is `Block.key`; unknown options are an error;
//   * int and float values are stored as std::to_string of the parsed number
//     (floats therefore keep 6 decimals) and parsed again when read;
//   * bools accept true/yes/on/1/TRUE/YES/ON and false/no/off/0/FALSE/NO/OFF;
//   * a key given twice keeps both values and readers take the first.
// The registered options are those of the five MDAS sample apps
// (optixMotionBlur.cpp:104-137 and siblings), so their .env files parse
// unchanged, plus a `Scene` block that selects this library's synthetic scenes.
#include <stdint.h>
#include <string.h>
#include <fstream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mdas.h"

namespace {

enum OptType { OPT_INT, OPT_FLOAT, OPT_BOOL, OPT_VECTOR3, OPT_VECTOR4, OPT_FRAME, OPT_PARALLELOGRAM, OPT_STRING };

struct Option {
    std::string name;
    OptType type;
    std::string defaultValue;
    std::vector<std::string> values;
};

// Number of value words each type consumes.
int arity(OptType t) {
    switch (t) {
        case OPT_VECTOR3: return 3;
        case OPT_VECTOR4: return 4;
        case OPT_FRAME: return 11;
        case OPT_PARALLELOGRAM: return 9;
        default: return 1;
    }
}

bool filter_value(const std::string& value, std::string& out, OptType type) {
    std::stringstream ss(value);
    switch (type) {
        case OPT_INT: {
            int v = 0;
            ss >> v;
            out = std::to_string(v);
            return true;
        }
        case OPT_FLOAT: {
            float v = 0.0f;
            ss >> v;
            out = std::to_string(v);
            return true;
        }
        case OPT_BOOL: {
            if (value == "true" || value == "yes" || value == "on" || value == "1" || value == "TRUE" ||
                value == "YES" || value == "ON") {
                out = "1";
                return true;
            }
            if (value == "false" || value == "no" || value == "off" || value == "0" || value == "FALSE" ||
                value == "NO" || value == "OFF") {
                out = "0";
                return true;
            }
            return false;
        }
        case OPT_STRING:
            out = value;
            return !value.empty();
        default: {
            const int n = arity(type);
            out.clear();
            for (int i = 0; i < n; ++i) {
                float v = 0.0f;
                ss >> v;
                if (i) out += " ";
                out += std::to_string(v);
            }
            return true;
        }
    }
}

struct Environment {
    std::vector<Option> options;

    void reg(const char* name, OptType type, const char* def = nullptr) {
        Option o;
        o.name = name;
        o.type = type;
        if (def) filter_value(def, o.defaultValue, type);
        options.push_back(o);
    }

    Environment() {
        reg("Camera.position", OPT_VECTOR3);
        reg("Camera.direction", OPT_VECTOR3);
        reg("Camera.upVector", OPT_VECTOR3, "0.0 1.0 0.0");
        reg("Camera.fovy", OPT_FLOAT, "45.0");
        reg("Camera.focalDistance", OPT_FLOAT, "0.0");
        reg("Camera.lensRadius", OPT_FLOAT, "0.0");
        reg("EnvironmentMap.filename", OPT_STRING);
        reg("Film.filename", OPT_STRING);
        reg("Film.width", OPT_INT, "1024");
        reg("Film.height", OPT_INT, "768");
        reg("Sampler.samples", OPT_FLOAT, "1");
        reg("Sampler.mdas", OPT_BOOL, "0");
        reg("Mdas.scaleFactor", OPT_FLOAT, "1.0");
        reg("Mdas.alpha", OPT_FLOAT, "0.25");
        reg("Mdas.bitsPerDim", OPT_INT, "0");
        reg("Mdas.extraImgBits", OPT_INT, "8");
        reg("Mdas.candidatesNum", OPT_INT, "4");
        reg("Light.point", OPT_VECTOR3);
        reg("Light.distant", OPT_VECTOR3);
        reg("Light.color", OPT_VECTOR3);
        reg("Light.area", OPT_PARALLELOGRAM);
        reg("Light.background", OPT_VECTOR3, "1.0 1.0 1.0");
        reg("Model.filename", OPT_STRING);
        reg("Model.frame", OPT_FRAME);
        reg("Model.emissive", OPT_BOOL, "0");
        reg("Scene.kind", OPT_STRING);
        reg("Scene.seed", OPT_INT, "0");
        reg("Scene.count", OPT_INT, "0");
    }

    Option* find(const std::string& name) {
        for (Option& o : options)
            if (o.name == name) return &o;
        return nullptr;
    }

    // first stored value, else the default (Environment.cpp:143-177)
    const std::string* raw(const char* name) {
        Option* o = find(name);
        if (!o) return nullptr;
        if (!o->values.empty() && !o->values.front().empty()) return &o->values.front();
        if (!o->defaultValue.empty()) return &o->defaultValue;
        return nullptr;
    }

    template <class T>
    bool get(const char* name, T& out) {
        const std::string* s = raw(name);
        if (!s) return false;
        std::stringstream ss(*s);
        ss >> out;
        return true;
    }

    bool read(const std::string& filename, std::string& err) {
        std::ifstream in(filename);
        if (!in.good()) {
            err = "Cannot open file '" + filename + "'!";
            return false;
        }
        std::string blockName, last, value, line;
        bool block = false;
        int lineNumber = 0;
        while (std::getline(in, line)) {
            ++lineNumber;
            const size_t comment = line.find('#');
            if (comment != std::string::npos) line = line.substr(0, comment);
            std::stringstream ss(line);
            std::vector<std::string> words{std::istream_iterator<std::string>{ss}, std::istream_iterator<std::string>{}};
            for (size_t i = 0; i < words.size(); ++i) {
                if (words[i] == "{") {
                    blockName = last;
                    block = true;
                } else if (words[i] == "}") {
                    if (blockName.empty()) {
                        err = "Unpaired } in '" + filename + "' (line " + std::to_string(lineNumber) + ").";
                        return false;
                    }
                    block = false;
                    blockName.clear();
                } else if (block) {
                    const std::string optionName = blockName + "." + words[i];
                    Option* o = find(optionName);
                    if (!o) {
                        err = "Unknown option '" + optionName + "' in environment file '" + filename + "' (line " +
                              std::to_string(lineNumber) + ").";
                        return false;
                    }
                    const int n = arity(o->type);
                    if (i + n >= words.size()) {
                        err = "Mismatch in variable " + optionName + " in environment file '" + filename +
                              "' (line " + std::to_string(lineNumber) + ").";
                        return false;
                    }
                    std::string joined = words[i + 1];
                    for (int k = 2; k <= n; ++k) joined += " " + words[i + k];
                    if (!filter_value(joined, value, o->type)) {
                        err = "Mismatch in variable " + optionName + " in environment file '" + filename +
                              "' (line " + std::to_string(lineNumber) + ").";
                        return false;
                    }
                    o->values.push_back(value);
                    i += n;
                }
                last = words[i];
            }
        }
        return true;
    }
};

int scene_kind_of(const std::string& s) {
    if (s == "mb" || s == "motionblur") return MDAS_SCENE_DISCS_MB;
    if (s == "dof" || s == "depthoffield") return MDAS_SCENE_DISCS_DOF;
    if (s == "mbdof") return MDAS_SCENE_DISCS_MBDOF;
    if (s == "dl" || s == "directlighting") return MDAS_SCENE_DIRECT_LIGHT;
    return -2;
}

void fill(Environment& env, mdas_config* cfg) {
    bool b = false;
    if (env.get("Sampler.mdas", b)) cfg->mdas = b ? 1 : 0;
    env.get("Sampler.samples", cfg->samples);
    env.get("Mdas.scaleFactor", cfg->scaleFactor);
    env.get("Mdas.alpha", cfg->alpha);
    env.get("Mdas.bitsPerDim", cfg->bitsPerDim);
    env.get("Mdas.extraImgBits", cfg->extraImgBits);
    env.get("Mdas.candidatesNum", cfg->candidatesNum);
    env.get("Film.width", cfg->width);
    env.get("Film.height", cfg->height);
    env.get("Camera.focalDistance", cfg->focalDistance);
    env.get("Camera.lensRadius", cfg->lensRadius);
    env.get("Camera.fovy", cfg->fovy);
    env.get("Scene.count", cfg->sceneCount);
    long long seed = 0;
    if (env.get("Scene.seed", seed)) cfg->sceneSeed = seed;
    const std::string* kind = env.raw("Scene.kind");
    cfg->sceneKind = kind ? scene_kind_of(*kind) : -1;
    const std::string* fn = env.raw("Film.filename");
    cfg->filmFilename[0] = 0;
    if (fn) {
        strncpy(cfg->filmFilename, fn->c_str(), sizeof(cfg->filmFilename) - 1);
        cfg->filmFilename[sizeof(cfg->filmFilename) - 1] = 0;
    }
}

}  // namespace

extern "C" {

int mdas_config_defaults(mdas_config* cfg) {
    if (!cfg) return MDAS_ERR_INVALID;
    memset(cfg, 0, sizeof(*cfg));
    Environment env;
    fill(env, cfg);
    return MDAS_OK;
}

int mdas_config_read(const char* path, mdas_config* cfg, char* err, int errBytes) {
    if (!path || !cfg) return MDAS_ERR_INVALID;
    memset(cfg, 0, sizeof(*cfg));
    Environment env;
    std::string e;
    if (!env.read(path, e)) {
        if (err && errBytes > 0) {
            strncpy(err, e.c_str(), (size_t)errBytes - 1);
            err[errBytes - 1] = 0;
        }
        return MDAS_ERR_INVALID;
    }
    fill(env, cfg);
    if (cfg->sceneKind == -2) {
        if (err && errBytes > 0) {
            strncpy(err, "Unknown Scene.kind", (size_t)errBytes - 1);
            err[errBytes - 1] = 0;
        }
        return MDAS_ERR_INVALID;
    }
    if (err && errBytes > 0) err[0] = 0;
    return MDAS_OK;
}

}  // extern "C"
