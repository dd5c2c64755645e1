// prm.h -- reader for the reference's input.prm format (deal.II ParameterHandler subset):
//   subsection <name> ... end   (nested)
//   set <key> = <value>         (# starts a comment; a trailing backslash continues the line)
// Entries must be declared (with a default) before parsing, as ParameterHandler requires.
#pragma once

#include <map>
#include <string>
#include <vector>

namespace plens {

class ParameterHandler {
public:
    // `path` is "sub/sub/key", e.g. "BCs/bid1/type".
    void declare_entry(const std::string& path, const std::string& default_value,
                       const std::string& doc = "");
    // Parses prm text; throws std::runtime_error naming the line of the first problem.
    void parse_input_from_string(const std::string& text);
    void parse_input(const std::string& filename);

    std::string get(const std::string& path) const;
    double get_double(const std::string& path) const;
    long get_integer(const std::string& path) const;
    bool get_bool(const std::string& path) const;
    bool was_set(const std::string& path) const;
    // Writes all entries with their current values in declaration order, as
    // ParameterHandler::print_parameters(..., KeepDeclarationOrder) does.
    std::string print_parameters() const;

private:
    struct Entry {
        std::string value, doc;
        bool set = false;
    };
    std::map<std::string, Entry> entries_;
    std::vector<std::string> order_;
};

// Splits `s` at `delim` and trims each piece (utilities/split_string.h:30-48).
std::vector<std::string> split_string(const std::string& s, const std::string& delim);
std::string trim(const std::string& s);

}  // namespace plens
