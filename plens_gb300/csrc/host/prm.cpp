// prm.cpp -- see prm.h.
#include "prm.h"

#include <algorithm>
#include <cctype>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace plens {

std::string trim(const std::string& s)
{
    size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    return s.substr(b, e - b);
}

std::vector<std::string> split_string(const std::string& s, const std::string& delim)
{
    std::vector<std::string> out;
    if (delim == " ") {
        std::istringstream is(s);
        std::string w;
        while (is >> w) out.push_back(w);
        return out;
    }
    size_t start = 0;
    for (;;) {
        const size_t p = s.find(delim, start);
        out.push_back(trim(s.substr(start, p == std::string::npos ? std::string::npos : p - start)));
        if (p == std::string::npos) break;
        start = p + delim.size();
    }
    return out;
}

void ParameterHandler::declare_entry(const std::string& path, const std::string& default_value,
                                     const std::string& doc)
{
    if (entries_.find(path) == entries_.end()) order_.push_back(path);
    entries_[path] = Entry{default_value, doc, false};
}

void ParameterHandler::parse_input_from_string(const std::string& text)
{
    // join continuation lines first
    std::vector<std::pair<int, std::string>> lines;
    {
        std::istringstream is(text);
        std::string raw, acc;
        int lineno = 0, start = 0;
        while (std::getline(is, raw)) {
            ++lineno;
            const size_t hash = raw.find('#');
            if (hash != std::string::npos) raw = raw.substr(0, hash);
            std::string t = trim(raw);
            if (acc.empty()) start = lineno;
            if (!t.empty() && t.back() == '\\') {
                t.pop_back();
                acc += t + " ";
                continue;
            }
            acc += t;
            lines.emplace_back(start, acc);
            acc.clear();
        }
        if (!acc.empty()) lines.emplace_back(start, acc);
    }
    std::vector<std::string> stack;
    for (const auto& [lineno, line] : lines) {
        if (line.empty()) continue;
        auto err = [&](const std::string& m) {
            throw std::runtime_error("input.prm line " + std::to_string(lineno) + ": " + m);
        };
        if (line.rfind("subsection", 0) == 0) {
            stack.push_back(trim(line.substr(10)));
            continue;
        }
        if (line == "end") {
            if (stack.empty()) err("'end' without subsection");
            stack.pop_back();
            continue;
        }
        if (line.rfind("set", 0) == 0) {
            const std::string rest = line.substr(3);
            const size_t eq = rest.find('=');
            if (eq == std::string::npos) err("'set' without '='");
            std::string key = trim(rest.substr(0, eq));
            std::string val = trim(rest.substr(eq + 1));
            std::string path;
            for (const auto& sub : stack) path += sub + "/";
            path += key;
            auto it = entries_.find(path);
            if (it == entries_.end()) err("undeclared entry '" + path + "'");
            it->second.value = val;
            it->second.set = true;
            continue;
        }
        err("cannot parse '" + line + "'");
    }
    if (!stack.empty()) throw std::runtime_error("input.prm: missing 'end' for subsection " + stack.back());
}

void ParameterHandler::parse_input(const std::string& filename)
{
    std::ifstream f(filename);
    if (!f.good()) throw std::runtime_error("cannot open parameter file " + filename);
    std::stringstream ss;
    ss << f.rdbuf();
    parse_input_from_string(ss.str());
}

std::string ParameterHandler::get(const std::string& path) const
{
    auto it = entries_.find(path);
    if (it == entries_.end()) throw std::runtime_error("undeclared entry '" + path + "'");
    return it->second.value;
}

double ParameterHandler::get_double(const std::string& path) const
{
    const std::string v = get(path);
    try {
        size_t used = 0;
        const double d = std::stod(v, &used);
        if (trim(v.substr(used)).size()) throw std::invalid_argument(v);
        return d;
    } catch (const std::exception&) {
        throw std::runtime_error("entry '" + path + "' is not a number: '" + v + "'");
    }
}

long ParameterHandler::get_integer(const std::string& path) const
{
    const std::string v = get(path);
    try {
        size_t used = 0;
        const long d = std::stol(v, &used);
        if (trim(v.substr(used)).size()) throw std::invalid_argument(v);
        return d;
    } catch (const std::exception&) {
        throw std::runtime_error("entry '" + path + "' is not an integer: '" + v + "'");
    }
}

bool ParameterHandler::get_bool(const std::string& path) const
{
    std::string v = get(path);
    std::transform(v.begin(), v.end(), v.begin(), [](unsigned char c) { return std::tolower(c); });
    if (v == "true" || v == "yes" || v == "1") return true;
    if (v == "false" || v == "no" || v == "0") return false;
    throw std::runtime_error("entry '" + path + "' is not a bool: '" + v + "'");
}

bool ParameterHandler::was_set(const std::string& path) const
{
    auto it = entries_.find(path);
    return it != entries_.end() && it->second.set;
}

std::string ParameterHandler::print_parameters() const
{
    std::ostringstream os;
    std::vector<std::string> open;
    for (const auto& path : order_) {
        std::vector<std::string> parts = split_string(path, "/");
        const std::string key = parts.back();
        parts.pop_back();
        size_t common = 0;
        while (common < open.size() && common < parts.size() && open[common] == parts[common])
            ++common;
        while (open.size() > common) {
            open.pop_back();
            os << std::string(2 * open.size(), ' ') << "end\n";
        }
        while (open.size() < parts.size()) {
            os << std::string(2 * open.size(), ' ') << "subsection " << parts[open.size()] << "\n";
            open.push_back(parts[open.size()]);
        }
        const Entry& e = entries_.at(path);
        if (!e.doc.empty()) os << std::string(2 * open.size(), ' ') << "# " << e.doc << "\n";
        os << std::string(2 * open.size(), ' ') << "set " << key << " = " << e.value << "\n";
    }
    while (!open.empty()) {
        open.pop_back();
        os << std::string(2 * open.size(), ' ') << "end\n";
    }
    return os.str();
}

}  // namespace plens
