/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The part of libconfig++ that the reference's configuration readers use
 * (c++/src/ConfigurationNetworkGrowth.cpp:7-120,
 * c++/src/ConfigurationNetworkTopology.cpp:7-45): Config::readFile,
 * Config::getRoot, Setting::operator[](name) for groups, Setting::lookupValue
 * and the exception types they catch.  The parser reads libconfig's
 * documented grammar for groups and scalars: `name = value;` or
 * `name : value;`, groups in braces, integers (decimal or 0x hex, optional L
 * suffix), floats, booleans, strings (adjacent literals concatenate), and the
 * three comment forms.  lookupValue follows libconfig's default of no
 * automatic number conversion: an integer setting does not fill a double and a
 * float setting does not fill an int (the lookup returns false and leaves the
 * value alone).
 */
#ifndef UG_REF_SHIM_LIBCONFIG_HPP
#define UG_REF_SHIM_LIBCONFIG_HPP

#include <cctype>
#include <cerrno>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace libconfig {

class ConfigException : public std::exception {
public:
    const char* what() const noexcept override { return "ConfigException"; }
};

class FileIOException : public ConfigException {
public:
    const char* what() const noexcept override { return "FileIOException"; }
};

class ParseException : public ConfigException {
public:
    ParseException(const std::string& file, int line, const std::string& error)
        : file_(file), line_(line), error_(error) {}
    const char* getFile() const { return file_.c_str(); }
    int getLine() const { return line_; }
    const char* getError() const { return error_.c_str(); }
    const char* what() const noexcept override { return "ParseException"; }

private:
    std::string file_;
    int line_;
    std::string error_;
};

class SettingNotFoundException : public ConfigException {
public:
    const char* what() const noexcept override { return "SettingNotFoundException"; }
};

class SettingTypeException : public ConfigException {
public:
    const char* what() const noexcept override { return "SettingTypeException"; }
};

class Setting {
public:
    enum Type { TypeNone, TypeInt, TypeInt64, TypeFloat, TypeString, TypeBoolean, TypeGroup };

    Setting() : type_(TypeGroup), i_(0), f_(0) {}

    Type getType() const { return type_; }
    bool isGroup() const { return type_ == TypeGroup; }

    const Setting& operator[](const char* name) const
    {
        const Setting* s = find(name);
        if (!s) throw SettingNotFoundException();
        return *s;
    }
    const Setting& operator[](const std::string& name) const { return (*this)[name.c_str()]; }
    bool exists(const char* name) const { return find(name) != nullptr; }

    bool lookupValue(const char* name, int& v) const
    {
        const Setting* s = find(name);
        if (!s || (s->type_ != TypeInt && s->type_ != TypeInt64)) return false;
        v = (int)s->i_;
        return true;
    }
    bool lookupValue(const char* name, long& v) const
    {
        const Setting* s = find(name);
        if (!s || (s->type_ != TypeInt && s->type_ != TypeInt64)) return false;
        v = (long)s->i_;
        return true;
    }
    bool lookupValue(const char* name, long long& v) const
    {
        const Setting* s = find(name);
        if (!s || (s->type_ != TypeInt && s->type_ != TypeInt64)) return false;
        v = s->i_;
        return true;
    }
    bool lookupValue(const char* name, unsigned& v) const
    {
        const Setting* s = find(name);
        if (!s || (s->type_ != TypeInt && s->type_ != TypeInt64)) return false;
        v = (unsigned)s->i_;
        return true;
    }
    bool lookupValue(const char* name, double& v) const
    {
        const Setting* s = find(name);
        if (!s || s->type_ != TypeFloat) return false;
        v = s->f_;
        return true;
    }
    bool lookupValue(const char* name, float& v) const
    {
        const Setting* s = find(name);
        if (!s || s->type_ != TypeFloat) return false;
        v = (float)s->f_;
        return true;
    }
    bool lookupValue(const char* name, bool& v) const
    {
        const Setting* s = find(name);
        if (!s || s->type_ != TypeBoolean) return false;
        v = s->i_ != 0;
        return true;
    }
    bool lookupValue(const char* name, std::string& v) const
    {
        const Setting* s = find(name);
        if (!s || s->type_ != TypeString) return false;
        v = s->s_;
        return true;
    }

private:
    friend class Config;

    const Setting* find(const char* name) const
    {
        if (type_ != TypeGroup) return nullptr;
        for (size_t k = 0; k < names_.size(); ++k)
            if (names_[k] == name) return children_[k].get();
        return nullptr;
    }

    Type type_;
    long long i_;
    double f_;
    std::string s_;
    std::vector<std::string> names_;
    std::vector<std::unique_ptr<Setting>> children_;
};

class Config {
public:
    Config() : root_(new Setting()) {}

    const Setting& getRoot() const { return *root_; }

    void readFile(const char* filename)
    {
        std::ifstream in(filename);
        if (!in) throw FileIOException();
        std::stringstream ss;
        ss << in.rdbuf();
        file_ = filename;
        text_ = ss.str();
        pos_ = 0;
        line_ = 1;
        root_.reset(new Setting());
        parse_group_body(*root_, true);
    }

private:
    void fail(const std::string& what) { throw ParseException(file_, line_, what); }

    void skip()
    {
        for (;;) {
            while (pos_ < text_.size() && std::isspace((unsigned char)text_[pos_])) {
                if (text_[pos_] == '\n') ++line_;
                ++pos_;
            }
            if (pos_ >= text_.size()) return;
            if (text_[pos_] == '#' || (text_[pos_] == '/' && pos_ + 1 < text_.size() && text_[pos_ + 1] == '/')) {
                while (pos_ < text_.size() && text_[pos_] != '\n') ++pos_;
            } else if (text_[pos_] == '/' && pos_ + 1 < text_.size() && text_[pos_ + 1] == '*') {
                size_t e = text_.find("*/", pos_ + 2);
                if (e == std::string::npos) fail("unterminated comment");
                for (size_t k = pos_; k < e; ++k)
                    if (text_[k] == '\n') ++line_;
                pos_ = e + 2;
            } else {
                return;
            }
        }
    }

    void parse_group_body(Setting& g, bool top)
    {
        for (;;) {
            skip();
            if (pos_ >= text_.size()) {
                if (!top) fail("unexpected end of file in group");
                return;
            }
            if (text_[pos_] == '}') {
                if (top) fail("unexpected '}'");
                ++pos_;
                return;
            }
            size_t start = pos_;
            if (!(std::isalpha((unsigned char)text_[pos_]) || text_[pos_] == '*')) fail("expected a setting name");
            while (pos_ < text_.size() &&
                   (std::isalnum((unsigned char)text_[pos_]) || text_[pos_] == '_' || text_[pos_] == '-' || text_[pos_] == '*'))
                ++pos_;
            std::string name = text_.substr(start, pos_ - start);
            skip();
            if (pos_ >= text_.size() || (text_[pos_] != '=' && text_[pos_] != ':')) fail("expected '=' or ':'");
            ++pos_;
            std::unique_ptr<Setting> s(new Setting());
            parse_value(*s);
            g.names_.push_back(name);
            g.children_.push_back(std::move(s));
            skip();
            if (pos_ < text_.size() && (text_[pos_] == ';' || text_[pos_] == ',')) ++pos_;
        }
    }

    void parse_value(Setting& s)
    {
        skip();
        if (pos_ >= text_.size()) fail("expected a value");
        char c = text_[pos_];
        if (c == '{') {
            ++pos_;
            s.type_ = Setting::TypeGroup;
            parse_group_body(s, false);
            return;
        }
        if (c == '"') {
            s.type_ = Setting::TypeString;
            while (pos_ < text_.size() && text_[pos_] == '"') {
                ++pos_;
                while (pos_ < text_.size() && text_[pos_] != '"') {
                    if (text_[pos_] == '\\' && pos_ + 1 < text_.size()) {
                        char e = text_[pos_ + 1];
                        s.s_ += e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'f' ? '\f' : e;
                        pos_ += 2;
                    } else {
                        if (text_[pos_] == '\n') ++line_;
                        s.s_ += text_[pos_++];
                    }
                }
                if (pos_ >= text_.size()) fail("unterminated string");
                ++pos_;
                skip();
            }
            return;
        }
        size_t start = pos_;
        while (pos_ < text_.size() && !std::isspace((unsigned char)text_[pos_]) && text_[pos_] != ';' &&
               text_[pos_] != ',' && text_[pos_] != '}')
            ++pos_;
        std::string tok = text_.substr(start, pos_ - start);
        std::string low;
        for (char ch : tok) low += (char)std::tolower((unsigned char)ch);
        if (low == "true" || low == "false") {
            s.type_ = Setting::TypeBoolean;
            s.i_ = low == "true";
            return;
        }
        bool is_float = false, is_hex = low.size() > 2 && (low.compare(0, 2, "0x") == 0 ||
                                                          low.compare(0, 3, "-0x") == 0 || low.compare(0, 3, "+0x") == 0);
        if (!is_hex)
            for (char ch : low)
                if (ch == '.' || ch == 'e') is_float = true;
        std::string num = tok;
        bool wide = false;
        if (!is_float)
            while (!num.empty() && (num.back() == 'L' || num.back() == 'l')) {
                num.pop_back();
                wide = true;
            }
        errno = 0;
        char* end = nullptr;
        if (is_float) {
            s.type_ = Setting::TypeFloat;
            s.f_ = std::strtod(num.c_str(), &end);
        } else {
            s.i_ = std::strtoll(num.c_str(), &end, 0);
            s.type_ = wide ? Setting::TypeInt64 : Setting::TypeInt;
        }
        if (num.empty() || end != num.c_str() + num.size() || errno == ERANGE) fail("bad value '" + tok + "'");
    }

    std::unique_ptr<Setting> root_;
    std::string file_, text_;
    size_t pos_ = 0;
    int line_ = 1;
};

} // namespace libconfig

#endif
