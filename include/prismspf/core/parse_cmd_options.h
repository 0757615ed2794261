// Command line of a PRISMS-PF application (reference: include/prismspf/core/parse_cmd_options.h):
// `./main -i parameters.prm`; without -i the file is parameters.prm.
#pragma once

#include <algorithm>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/utilities/utilities.h>

PRISMS_PF_BEGIN_NAMESPACE

class ParseCMDOptions {
 public:
  ParseCMDOptions(int& _argc, char** argv) : argc(_argc) {
    for (int i = 1; i < argc; ++i) tokens.emplace_back(argv[i]);
  }

  std::string get_parameters_filename() {
    const int n_args = 3;
    if (argc > n_args)
      throw std::runtime_error(
          "Too many command line arguments. The arguments should specify the input file name, for example, "
          "`./main -i parameters.prm`");
    std::string file = "parameters.prm";
    if (argc >= n_args - 1 && !cmd_option_exists("-i"))
      throw std::runtime_error("Invalid command line option. Use `-i` to specify the input file, e.g., `./main -i "
                               "parameters.prm`.");
    if (cmd_option_exists("-i")) file = get_cmd_option("-i");
    if (file.size() < 4 || file.substr(file.size() - 4) != ".prm")
      throw std::runtime_error("The input file must have the `.prm` extension. Please rename the file accordingly.");
    if (!std::ifstream(file)) throw std::runtime_error("The specified parameters file `" + file + "` does not exist.");
    std::cout << "Using parameter file " << file << std::endl;
    return file;
  }

 private:
  bool cmd_option_exists(const std::string& o) const { return std::find(tokens.begin(), tokens.end(), o) != tokens.end(); }
  std::string get_cmd_option(const std::string& o) const {
    auto it = std::find(tokens.begin(), tokens.end(), o);
    if (it != tokens.end() && ++it != tokens.end()) return *it;
    return "";
  }
  int argc;
  std::vector<std::string> tokens;
};

PRISMS_PF_END_NAMESPACE
