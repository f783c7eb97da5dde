// Minimal command-line parser accepting the reference drivers' flag syntax
// (--name value, --name=value, boolean --flag), with unknown flags rejected.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <string>

namespace nbpg_cli {

struct Flags {
    std::map<std::string, std::function<void(const std::string &)>> opts;
    std::map<std::string, bool *> bools;
    void opt(const std::string &n, std::string &v) { opts[n] = [&v](const std::string &s) { v = s; }; }
    void opt(const std::string &n, uint32_t &v) { opts[n] = [&v](const std::string &s) { v = uint32_t(std::stoul(s)); }; }
    void opt(const std::string &n, uint64_t &v) { opts[n] = [&v](const std::string &s) { v = std::stoull(s); }; }
    void opt(const std::string &n, int &v) { opts[n] = [&v](const std::string &s) { v = std::stoi(s); }; }
    void opt(const std::string &n, double &v) { opts[n] = [&v](const std::string &s) { v = std::stod(s); }; }
    void opt(const std::string &n, float &v) { opts[n] = [&v](const std::string &s) { v = std::stof(s); }; }
    void flag(const std::string &n, bool &v) { bools[n] = &v; }

    // returns false (after printing why) on an unknown flag or a missing value
    bool parse(int argc, char **argv)
    {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a.rfind("--", 0) != 0) { std::fprintf(stderr, "unexpected argument: %s\n", a.c_str()); return false; }
            std::string name = a, val;
            bool has_val = false;
            auto eq = a.find('=');
            if (eq != std::string::npos) { name = a.substr(0, eq); val = a.substr(eq + 1); has_val = true; }
            if (bools.count(name)) { *bools[name] = has_val ? (val != "0" && val != "false") : true; continue; }
            if (!opts.count(name)) { std::fprintf(stderr, "The following argument was not expected: %s\n", name.c_str()); return false; }
            if (!has_val) {
                if (i + 1 >= argc) { std::fprintf(stderr, "%s requires a value\n", name.c_str()); return false; }
                val = argv[++i];
            }
            try { opts[name](val); } catch (...) { std::fprintf(stderr, "bad value for %s: %s\n", name.c_str(), val.c_str()); return false; }
        }
        return true;
    }
};

inline bool ends_with(const std::string &s, const std::string &suf)
{
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

}  // namespace nbpg_cli
