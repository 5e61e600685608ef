// options.h -- command-line handling shared by the drivers, with the reference
// parser's observable behaviour (cxx/CmdLineArgParser.cpp): `-name value`
// options and toggling flags; a token that is not an option (such as the
// positional "32 10" of the upwindCxx ctest cases) is ignored; an unknown
// -option prints "<arg> is not a valid option." and parsing fails.
#ifndef FDB_DRIVERS_OPTIONS_H
#define FDB_DRIVERS_OPTIONS_H

#include <cctype>
#include <iostream>
#include <map>
#include <string>

namespace fdb_drivers {

struct Options {
  std::map<std::string, std::string> values;  // valued options
  std::map<std::string, bool> flags;          // toggles
  std::map<std::string, std::string> help;
};

inline bool is_option_name(const std::string& a) {
  return a.size() >= 2 && a[0] == '-' && !std::isdigit((unsigned char)a[1]);
}

inline bool parse(Options& o, int argc, char** argv) {
  for (int a = 1; a < argc; ++a) {
    std::string arg(argv[a]);
    if (is_option_name(arg) && !o.values.count(arg) && !o.flags.count(arg)) {
      std::cout << arg << " is not a valid option.\n";
      return false;
    }
  }
  for (int a = 1; a < argc; ++a) {
    std::string arg(argv[a]);
    if (o.values.count(arg) && a + 1 < argc) o.values[arg] = argv[a + 1];
    if (o.flags.count(arg)) o.flags[arg] = !o.flags[arg];
  }
  return true;
}

inline void print_help(const Options& o, const char* purpose, const char* exe) {
  std::cout << purpose << "\n";
  std::cout << exe << " [options]\nUsage:\n";
  for (const auto& kv : o.values)
    std::cout << "\t" << kv.first << " <value> " << o.help.at(kv.first) << " (" << kv.second
              << ")\n";
  for (const auto& kv : o.flags)
    std::cout << "\t" << kv.first << ' ' << o.help.at(kv.first) << " (" << kv.second << ")\n";
}

}  // namespace fdb_drivers

#endif  // FDB_DRIVERS_OPTIONS_H
