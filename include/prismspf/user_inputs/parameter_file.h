// Reader of deal.II ParameterHandler input files (.prm) as PRISMS-PF writes them:
//   set <name> = <value>        an entry (value runs to the end of the line; '#' starts a
//                               comment; a trailing '\' joins the next line)
//   subsection <name> ... end   nesting
// Entries are stored under their subsection path ("output/number"). Names match after
// collapsing runs of blanks. "set Model constant <name> = ..." lines are kept apart for
// UserConstants (reference: user_constants.h:967-1000 scans the file for them the same way).
#pragma once

#include <cctype>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <prismspf/config.h>

PRISMS_PF_BEGIN_NAMESPACE

namespace prm {

inline std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}

inline std::string collapse_blanks(const std::string& s) {
  std::string out;
  bool blank = false;
  for (char ch : trim(s)) {
    if (std::isspace(static_cast<unsigned char>(ch))) {
      blank = true;
      continue;
    }
    if (blank && !out.empty()) out += ' ';
    blank = false;
    out += ch;
  }
  return out;
}

// comma-separated list, each item trimmed; empty input gives an empty list
inline std::vector<std::string> split_list(const std::string& s, char sep = ',') {
  std::vector<std::string> out;
  if (trim(s).empty()) return out;
  std::string item;
  std::istringstream in(s);
  while (std::getline(in, item, sep)) out.push_back(trim(item));
  return out;
}

inline double to_double(const std::string& s) {
  size_t pos = 0;
  const double v = std::stod(trim(s), &pos);
  if (trim(s).size() != pos) throw std::invalid_argument("not a number: " + s);
  return v;
}

inline int to_int(const std::string& s) {
  size_t pos = 0;
  const int v = std::stoi(trim(s), &pos);
  if (trim(s).size() != pos) throw std::invalid_argument("not an integer: " + s);
  return v;
}

inline bool to_bool(const std::string& s) {
  const std::string t = trim(s);
  if (t == "true" || t == "True" || t == "TRUE" || t == "yes" || t == "1") return true;
  if (t == "false" || t == "False" || t == "FALSE" || t == "no" || t == "0") return false;
  throw std::invalid_argument("not a bool: " + s);
}

class ParameterFile {
 public:
  ParameterFile() = default;
  explicit ParameterFile(const std::string& file_name) { read(file_name); }

  void read(const std::string& file_name) {
    std::ifstream in(file_name);
    if (!in) throw std::runtime_error("cannot open parameter file " + file_name);
    std::stringstream ss;
    ss << in.rdbuf();
    parse(ss.str(), file_name);
  }

  void parse(const std::string& text, const std::string& origin = "<string>") {
    std::vector<std::string> path;
    std::istringstream in(text);
    std::string raw, line;
    int lineno = 0;
    while (std::getline(in, raw)) {
      ++lineno;
      const size_t hash = raw.find('#');
      if (hash != std::string::npos) raw = raw.substr(0, hash);
      raw = trim(raw);
      if (!raw.empty() && raw.back() == '\\') {
        line += raw.substr(0, raw.size() - 1) + " ";
        continue;
      }
      line += raw;
      const std::string l = trim(line);
      line.clear();
      if (l.empty()) continue;
      if (starts_with_word(l, "subsection")) {
        path.push_back(collapse_blanks(l.substr(10)));
      } else if (l == "end") {
        if (path.empty()) throw std::runtime_error(origin + ":" + std::to_string(lineno) + ": unmatched 'end'");
        path.pop_back();
      } else if (starts_with_word(l, "set")) {
        const size_t eq = l.find('=');
        if (eq == std::string::npos)
          throw std::runtime_error(origin + ":" + std::to_string(lineno) + ": 'set' without '='");
        const std::string name = collapse_blanks(l.substr(3, eq - 3));
        const std::string value = trim(l.substr(eq + 1));
        if (path.empty() && name.rfind("Model constant ", 0) == 0) {
          model_constants[collapse_blanks(name.substr(15))] = value;
          constant_order.push_back(collapse_blanks(name.substr(15)));
        } else {
          entries[key(path, name)] = value;
        }
      } else {
        throw std::runtime_error(origin + ":" + std::to_string(lineno) + ": cannot parse '" + l + "'");
      }
    }
    if (!path.empty()) throw std::runtime_error(origin + ": subsection '" + path.back() + "' is not closed");
  }

  // value of `name` (or the first alias present) inside `section` ("" = top level)
  bool find(const std::string& section, const std::vector<std::string>& names, std::string& out) const {
    for (const auto& n : names) {
      auto it = entries.find(section.empty() ? n : section + "/" + n);
      if (it != entries.end()) {
        used.insert(it->first);
        out = it->second;
        return true;
      }
    }
    return false;
  }
  std::string get(const std::string& section, const std::vector<std::string>& names, const std::string& def) const {
    std::string v;
    return find(section, names, v) ? v : def;
  }

  // subsections of the top level whose name starts with `prefix` ("boundary conditions: ")
  std::vector<std::string> subsections_with_prefix(const std::string& prefix) const {
    std::set<std::string> out;
    for (const auto& [k, v] : entries) {
      const size_t slash = k.find('/');
      if (slash == std::string::npos) continue;
      const std::string sec = k.substr(0, slash);
      if (sec.rfind(prefix, 0) == 0) out.insert(sec);
    }
    return {out.begin(), out.end()};
  }

  // entries nobody asked for (after all reads): names this build does not know
  std::vector<std::string> unused() const {
    std::vector<std::string> out;
    for (const auto& [k, v] : entries)
      if (!used.count(k)) out.push_back(k);
    return out;
  }
  void mark_used_prefix(const std::string& prefix) const {
    for (const auto& [k, v] : entries)
      if (k.rfind(prefix, 0) == 0) used.insert(k);
  }

  std::map<std::string, std::string> entries;
  std::map<std::string, std::string> model_constants;
  std::vector<std::string> constant_order;

 private:
  static bool starts_with_word(const std::string& l, const char* w) {
    const std::string s(w);
    return l.size() > s.size() && l.compare(0, s.size(), s) == 0 && std::isspace(static_cast<unsigned char>(l[s.size()]));
  }
  static std::string key(const std::vector<std::string>& path, const std::string& name) {
    std::string k;
    for (const auto& p : path) k += p + "/";
    return k + name;
  }
  mutable std::set<std::string> used;
};

}  // namespace prm

PRISMS_PF_END_NAMESPACE
