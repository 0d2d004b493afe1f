// Test-infrastructure shim, written for this project: the subset of
// Boost.program_options that the reference's src/ffr_img.cpp uses, so that
// file compiles and runs unmodified in the oracle (Boost is not installed).
//
// Supported: options_description("caption").add_options()(names, help)
// (names "long,s"; no value = a presence flag), value<T>() with required()
// and default_value(v), bool_switch(), command_line_parser(argc, argv)
// .options(d).run(), store(parsed, variables_map), variables_map count /
// empty / find / end / operator[] and variable_value::as<T>() for string,
// vector<string>, bool and arithmetic T, and printing a description.
// Accepted forms: --long value, --long=value, -s value, -svalue.
#pragma once

#include <map>
#include <memory>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace boost::program_options {

class value_semantic
{
public:
    bool is_switch = false;
    bool is_multi = false;
    bool has_default = false;
    std::string default_text;
    value_semantic* required() { return this; }
    template <typename T>
    value_semantic* default_value(const T& v)
    {
        std::ostringstream os;
        os.precision(17);
        os << v;
        default_text = os.str();
        has_default = true;
        return this;
    }
};

template <typename T>
value_semantic* value()
{
    auto* v = new value_semantic;
    v->is_multi = std::is_same_v<T, std::vector<std::string>>;
    return v;
}

inline value_semantic* bool_switch()
{
    auto* v = new value_semantic;
    v->is_switch = true;
    v->has_default = true;
    v->default_text = "0";
    return v;
}

struct option
{
    std::string name, help;
    char shrt = 0;
    std::shared_ptr<value_semantic> sem;    // null: a presence flag
};

class options_description;

class options_adder
{
    options_description* d_;

public:
    explicit options_adder(options_description* d) : d_(d) {}
    options_adder& operator()(const char* names, const char* help);
    options_adder& operator()(const char* names, value_semantic* v, const char* help);
};

class options_description
{
public:
    std::string caption;
    std::vector<option> opts;
    explicit options_description(const std::string& c) : caption(c) {}
    options_adder add_options() { return options_adder(this); }
    void add(const char* names, value_semantic* v, const char* help)
    {
        option o;
        std::string n = names;
        const size_t comma = n.find(',');
        o.name = n.substr(0, comma);
        if (comma != std::string::npos && comma + 1 < n.size())
            o.shrt = n[comma + 1];
        o.help = help;
        o.sem.reset(v);
        opts.push_back(o);
    }
};

inline options_adder& options_adder::operator()(const char* names, const char* help)
{
    d_->add(names, nullptr, help);
    return *this;
}

inline options_adder& options_adder::operator()(const char* names, value_semantic* v,
                                                const char* help)
{
    d_->add(names, v, help);
    return *this;
}

inline std::ostream& operator<<(std::ostream& os, const options_description& d)
{
    os << d.caption << ":\n";
    for (const option& o : d.opts)
    {
        os << "  ";
        if (o.shrt)
            os << "-" << o.shrt << " [ --" << o.name << " ]";
        else
            os << "--" << o.name;
        if (o.sem && !o.sem->is_switch)
            os << " arg";
        os << "  " << o.help << "\n";
    }
    return os;
}

class variable_value
{
public:
    std::vector<std::string> vals;
    template <typename T>
    T as() const
    {
        if (vals.empty())
            throw std::runtime_error("program_options shim: option has no value");
        if constexpr (std::is_same_v<T, std::vector<std::string>>)
            return vals;
        else if constexpr (std::is_same_v<T, std::string>)
            return vals.back();
        else if constexpr (std::is_same_v<T, bool>)
            return vals.back() == "1";
        else
        {
            std::istringstream is(vals.back());
            T x{};
            if (!(is >> x) || !is.eof())
                throw std::runtime_error("the argument ('" + vals.back() + "') is invalid");
            return x;
        }
    }
};

class variables_map : public std::map<std::string, variable_value>
{
};

struct parsed_options
{
    std::vector<std::pair<std::string, std::string>> items;   // (long name, value)
    const options_description* desc = nullptr;
};

class command_line_parser
{
    std::vector<std::string> args_;
    const options_description* desc_ = nullptr;

public:
    command_line_parser(int argc, char** argv) : args_(argv + 1, argv + argc) {}
    command_line_parser& options(const options_description& d)
    {
        desc_ = &d;
        return *this;
    }
    parsed_options run() const
    {
        parsed_options p;
        p.desc = desc_;
        for (size_t k = 0; k < args_.size(); ++k)
        {
            const std::string& tok = args_[k];
            const option* o = nullptr;
            std::string val;
            bool have = false;
            if (tok.rfind("--", 0) == 0)
            {
                std::string n = tok.substr(2);
                const size_t eq = n.find('=');
                if (eq != std::string::npos)
                {
                    val = n.substr(eq + 1);
                    n = n.substr(0, eq);
                    have = true;
                }
                for (const option& c : desc_->opts)
                    if (c.name == n)
                        o = &c;
            }
            else if (tok.size() >= 2 && tok[0] == '-')
            {
                for (const option& c : desc_->opts)
                    if (c.shrt == tok[1])
                        o = &c;
                if (tok.size() > 2)
                {
                    val = tok.substr(2);
                    have = true;
                }
            }
            if (!o)
                throw std::runtime_error("unrecognised option '" + tok + "'");
            if (!o->sem || o->sem->is_switch)
            {
                p.items.emplace_back(o->name, "1");
                continue;
            }
            if (!have)
            {
                if (k + 1 >= args_.size())
                    throw std::runtime_error("the required argument for option '--" + o->name
                                             + "' is missing");
                val = args_[++k];
            }
            p.items.emplace_back(o->name, val);
        }
        return p;
    }
};

inline void store(const parsed_options& p, variables_map& vm)
{
    for (const auto& [name, val] : p.items)
        vm[name].vals.push_back(val);
    if (!p.desc)
        return;
    for (const option& o : p.desc->opts)
        if (o.sem && o.sem->has_default && vm.find(o.name) == vm.end())
            vm[o.name].vals.push_back(o.sem->default_text);
}

} // namespace boost::program_options
