// Minimal "--name=value" / "--name value" command-line parser for the
// miniapp programs (the reference uses the third-party cxxopts; only its
// behaviour for these flags is reproduced: defaults, ints, doubles and
// booleans written as true/false/1/0, and --help).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

struct Args {
    struct Opt {
        std::string help, value;
    };
    std::string prog, desc;
    std::vector<std::string> order;
    std::map<std::string, Opt> opts;
    bool help = false;

    Args(std::string p, std::string d) : prog(std::move(p)), desc(std::move(d)) {}
    void add(const std::string& name, const std::string& help_text, const std::string& def) {
        order.push_back(name);
        opts[name] = Opt{help_text, def};
    }
    void parse(int argc, const char** argv) {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a.rfind("--", 0) != 0) throw std::invalid_argument("unexpected argument " + a);
            a = a.substr(2);
            std::string name = a, value;
            bool has_value = false;
            const size_t eq = a.find('=');
            if (eq != std::string::npos) {
                name = a.substr(0, eq);
                value = a.substr(eq + 1);
                has_value = true;
            }
            if (name == "help") {
                help = true;
                continue;
            }
            auto it = opts.find(name);
            if (it == opts.end()) throw std::invalid_argument("unknown option --" + name);
            if (!has_value) {
                const bool is_bool = it->second.value == "true" || it->second.value == "false";
                if (is_bool && (i + 1 >= argc || std::string(argv[i + 1]).rfind("--", 0) == 0)) {
                    value = "true";
                } else {
                    if (i + 1 >= argc) throw std::invalid_argument("missing value for --" + name);
                    value = argv[++i];
                }
            }
            it->second.value = value;
        }
    }
    int i(const std::string& n) const { return std::stoi(opts.at(n).value); }
    double d(const std::string& n) const { return std::stod(opts.at(n).value); }
    std::string s(const std::string& n) const { return opts.at(n).value; }
    bool b(const std::string& n) const {
        const std::string& v = opts.at(n).value;
        if (v == "true" || v == "1") return true;
        if (v == "false" || v == "0") return false;
        throw std::invalid_argument("bad boolean for --" + n + ": " + v);
    }
    void print_help() const {
        printf("%s\n  %s\n\n", desc.c_str(), prog.c_str());
        for (auto& n : order) printf("  --%-18s %s (default: %s)\n", n.c_str(), opts.at(n).help.c_str(), opts.at(n).value.c_str());
    }
};
