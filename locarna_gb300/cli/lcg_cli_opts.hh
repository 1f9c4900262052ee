// Command-line option table of the locarna / locarna_p drivers: GNU-style
// long options (--name value, --name=value), single-letter short options, and
// positional arguments, with the value kinds of the reference's option
// definitions (src/LocARNA/options.hh: O_NO_ARG, O_ARG_INT, O_ARG_DOUBLE,
// O_ARG_STRING, O_ARG_BOOL). Options the reference knows but this build does
// not implement are registered as unsupported and refused with an error.
#pragma once
#include <cstdlib>
#include <string>
#include <vector>

#ifndef LCG_CLI_PACKAGE_STRING
#define LCG_CLI_PACKAGE_STRING "LocARNA 2.0.1"
#endif

namespace lcg_cli {

class OptionTable {
    enum Kind { FLAG, INT, REAL, STR, BOOL, UNSUP };
    struct Opt {
        std::string name;
        char short_name;
        Kind kind;
        void *target;
        bool *given;
    };
    std::vector<Opt> opts_;
    std::string prog_, what_;

    void add(const std::string &n, char s, Kind k, void *t, bool *g) { opts_.push_back({n, s, k, t, g}); }

    static bool parse_bool(const std::string &v, bool &out) {
        if (v == "true" || v == "1" || v == "on" || v == "yes") out = true;
        else if (v == "false" || v == "0" || v == "off" || v == "no") out = false;
        else return false;
        return true;
    }

    bool assign(const Opt &o, const std::string &v, std::string &err) {
        char *end = nullptr;
        switch (o.kind) {
        case INT: {
            long x = std::strtol(v.c_str(), &end, 10);
            if (v.empty() || *end) {
                err = "Option --" + o.name + " expects an integer, got '" + v + "'.";
                return false;
            }
            *(int *)o.target = (int)x;
            break;
        }
        case REAL: {
            double x = std::strtod(v.c_str(), &end);
            if (v.empty() || *end) {
                err = "Option --" + o.name + " expects a number, got '" + v + "'.";
                return false;
            }
            *(double *)o.target = x;
            break;
        }
        case STR: *(std::string *)o.target = v; break;
        case BOOL:
            if (!parse_bool(v, *(bool *)o.target)) {
                err = "Option --" + o.name + " expects true or false, got '" + v + "'.";
                return false;
            }
            break;
        default: break;
        }
        if (o.given) *o.given = true;
        return true;
    }

public:
    OptionTable(std::string prog, std::string what) : prog_(std::move(prog)), what_(std::move(what)) {}
    void flag(const std::string &n, char s, bool *t) { add(n, s, FLAG, t, nullptr); }
    void integer(const std::string &n, char s, int *t, bool *given = nullptr) { add(n, s, INT, t, given); }
    void real(const std::string &n, char s, double *t, bool *given = nullptr) { add(n, s, REAL, t, given); }
    void string(const std::string &n, char s, std::string *t, bool *given = nullptr) { add(n, s, STR, t, given); }
    void boolean(const std::string &n, char s, bool *t, bool *given = nullptr) { add(n, s, BOOL, t, given); }
    void unsupported(const std::string &n) { add(n, 0, UNSUP, nullptr, nullptr); }

    bool parse(int argc, char **argv, std::vector<std::string> &positional, std::string &err) {
        for (int k = 1; k < argc; ++k) {
            std::string a = argv[k];
            const Opt *o = nullptr;
            std::string val;
            bool has_val = false;
            if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
                std::string name = a.substr(2);
                const size_t eq = name.find('=');
                if (eq != std::string::npos) {
                    val = name.substr(eq + 1);
                    name = name.substr(0, eq);
                    has_val = true;
                }
                for (const auto &x : opts_)
                    if (x.name == name) o = &x;
                if (!o) {
                    err = "Unknown option --" + name + ".";
                    return false;
                }
            } else if (a.size() == 2 && a[0] == '-' && a[1] != '-') {
                for (const auto &x : opts_)
                    if (x.short_name == a[1]) o = &x;
                if (!o) {
                    err = "Unknown option " + a + ".";
                    return false;
                }
            } else {
                positional.push_back(a);
                continue;
            }
            if (o->kind == UNSUP) {
                err = "Option --" + o->name + " of the reference is not supported by this build.";
                return false;
            }
            if (o->kind == FLAG) {
                if (has_val) {
                    err = "Option --" + o->name + " takes no value.";
                    return false;
                }
                *(bool *)o->target = true;
                continue;
            }
            if (!has_val) {
                if (k + 1 >= argc) {
                    err = "Option --" + o->name + " needs a value.";
                    return false;
                }
                val = argv[++k];
            }
            if (!assign(*o, val, err)) return false;
        }
        return true;
    }

    std::string usage() const {
        std::string u = "Usage: " + prog_ + " [options] <file 1> <file 2>\n" + what_ + "\nOptions:\n";
        for (const auto &o : opts_) {
            if (o.kind == UNSUP) continue;
            u += "  --" + o.name;
            if (o.short_name) u += std::string(", -") + o.short_name;
            switch (o.kind) {
            case INT: u += " <int>"; break;
            case REAL: u += " <number>"; break;
            case STR: u += " <string>"; break;
            case BOOL: u += " <bool>"; break;
            default: break;
            }
            u += "\n";
        }
        return u;
    }
};

}  // namespace lcg_cli
