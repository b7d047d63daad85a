// Shared pieces of the command-line drivers: the reference's option parser
// (src/parseCommandLine.hpp:4-37) and a wall-clock timer in seconds
// (src/get_time.hpp).
#pragma once
#include <sys/time.h>

#include <cstdlib>
#include <string>

struct CommandLine {
  int argc;
  char** argv;
  bool getOption(const std::string& o) const {
    for (int i = 1; i < argc; i++)
      if (o == argv[i]) return true;
    return false;
  }
  const char* getOptionValue(const std::string& o) const {
    for (int i = 1; i + 1 < argc; i++)
      if (o == argv[i]) return argv[i + 1];
    return nullptr;
  }
  long getOptionInt(const std::string& o, long d) const {
    const char* s = getOptionValue(o);
    return s ? std::atol(s) : d;
  }
  double getOptionDouble(const std::string& o, double d) const {
    const char* s = getOptionValue(o);
    return s ? std::atof(s) : d;
  }
};

inline double wall_seconds() {
  timeval t;
  gettimeofday(&t, nullptr);
  return t.tv_sec + t.tv_usec / 1e6;
}
