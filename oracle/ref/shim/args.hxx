// Minimal stand-in for the subset of the args flag library the reference's
// option classes use (include/option.hpp: ArgumentParser, HelpFlag,
// ValueFlag<T>, args::get, Help / ParseError / ValidationError, and printing
// the parser).  Written from those call sites: flags are matched by
// "-x value", "-xvalue", "--name value" or "--name=value".  Test
// infrastructure for building the reference baseline.
#pragma once
// The real header pulls these in; the reference relies on them transitively.
#include <algorithm>
#include <array>
#include <cstdint>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <memory>
#include <unordered_map>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace args {

struct Error : std::runtime_error {
    explicit Error(const std::string &s) : std::runtime_error(s) {}
};
struct Help : Error {
    explicit Help(const std::string &s) : Error(s) {}
};
struct ParseError : Error {
    explicit ParseError(const std::string &s) : Error(s) {}
};
struct ValidationError : Error {
    explicit ValidationError(const std::string &s) : Error(s) {}
};

struct EitherFlag {
    bool is_short;
    char s;
    std::string l;
    EitherFlag(char c) : is_short(true), s(c) {}
    EitherFlag(const char *x) : is_short(false), s(0), l(x) {}
};

class ArgumentParser;

class FlagBase {
public:
    std::string name, help;
    std::vector<EitherFlag> keys;
    bool matched = false;
    FlagBase(ArgumentParser &p, const std::string &n, const std::string &h,
             std::initializer_list<EitherFlag> k);
    virtual ~FlagBase() {}
    virtual bool takes_value() const = 0;
    virtual void set(const std::string &v) = 0;
    explicit operator bool() const { return matched; }
    std::string spelling() const
    {
        std::string out;
        for (const auto &k : keys) {
            if (!out.empty()) out += ", ";
            out += k.is_short ? std::string("-") + k.s : "--" + k.l;
        }
        return out;
    }
};

class ArgumentParser {
public:
    std::string desc, epilog;
    std::vector<FlagBase *> flags;
    ArgumentParser(const std::string &d, const std::string &e = "") : desc(d), epilog(e) {}
    void add(FlagBase *f) { flags.push_back(f); }
    FlagBase *find_short(char c)
    {
        for (auto *f : flags)
            for (const auto &k : f->keys)
                if (k.is_short && k.s == c) return f;
        return nullptr;
    }
    FlagBase *find_long(const std::string &l)
    {
        for (auto *f : flags)
            for (const auto &k : f->keys)
                if (!k.is_short && k.l == l) return f;
        return nullptr;
    }
    void ParseCLI(int argc, const char *const *argv)
    {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            FlagBase *f = nullptr;
            std::string val;
            bool have_val = false;
            if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
                std::string body = a.substr(2);
                const size_t eq = body.find('=');
                if (eq != std::string::npos) {
                    val = body.substr(eq + 1);
                    body = body.substr(0, eq);
                    have_val = true;
                }
                f = find_long(body);
            } else if (a.size() >= 2 && a[0] == '-') {
                f = find_short(a[1]);
                if (a.size() > 2) {
                    val = a.substr(2);
                    have_val = true;
                }
            }
            if (!f) throw ParseError("Flag could not be matched: " + a);
            if (f->takes_value() && !have_val) {
                if (i + 1 >= argc) throw ParseError("Flag '" + a + "' requires an argument");
                val = argv[++i];
            }
            f->matched = true;
            f->set(val);
        }
    }
};

inline FlagBase::FlagBase(ArgumentParser &p, const std::string &n, const std::string &h,
                          std::initializer_list<EitherFlag> k)
    : name(n), help(h), keys(k)
{
    p.add(this);
}

inline std::ostream &operator<<(std::ostream &os, const ArgumentParser &p)
{
    os << p.desc << "\n";
    for (const auto *f : p.flags) os << "  " << f->spelling() << "  " << f->help << "\n";
    return os << p.epilog;
}

class HelpFlag : public FlagBase {
public:
    HelpFlag(ArgumentParser &p, const std::string &n, const std::string &h,
             std::initializer_list<EitherFlag> k)
        : FlagBase(p, n, h, k)
    {
    }
    bool takes_value() const override { return false; }
    void set(const std::string &) override { throw Help(name); }
};

template <typename T> class ValueFlag : public FlagBase {
public:
    T value{};
    ValueFlag(ArgumentParser &p, const std::string &n, const std::string &h,
              std::initializer_list<EitherFlag> k)
        : FlagBase(p, n, h, k)
    {
    }
    bool takes_value() const override { return true; }
    void set(const std::string &v) override
    {
        std::istringstream is(v);
        if (!(is >> value)) throw ParseError("Argument '" + name + "' received invalid value '" + v + "'");
    }
};

template <> inline void ValueFlag<std::string>::set(const std::string &v) { value = v; }

template <> inline void ValueFlag<uint16_t>::set(const std::string &v)
{
    std::istringstream is(v);
    unsigned long x = 0;
    if (!(is >> x) || x > 0xFFFFul) throw ParseError("Argument '" + name + "' received invalid value '" + v + "'");
    value = (uint16_t)x;
}

template <typename T> T &get(ValueFlag<T> &f) { return f.value; }

}  // namespace args
