// Host-side helpers shared by the C-ABI implementation files.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "omc_gpu.h"

namespace omc {

constexpr double kRM = 0.5109989461;  // MeV, ompMC ompmc.h:46

// Records a formatted message as this thread's last error and returns s.
omc_status fail(omc_status s, const char *fmt, ...);
void clear_error();

// Reads a whole file; false if it cannot be opened.
bool read_file(const std::string &path, std::string &out);

// Splits text into lines (without the trailing newline characters).
std::vector<std::string> split_lines(const std::string &text);

// Removes every white-space character (removeSpaces, omc_utilities.c:144).
std::string remove_spaces(const std::string &s);

// Whitespace-separated number stream over a block of text.
class NumberStream {
 public:
  explicit NumberStream(const char *p) : p_(p) {}
  bool next(double &v);
  bool next_int(int &v);
  const char *pos() const { return p_; }

 private:
  const char *p_;
};

}  // namespace omc
