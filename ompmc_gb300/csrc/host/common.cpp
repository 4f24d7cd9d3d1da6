#include "common.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace omc {

static thread_local std::string g_last_error;

omc_status fail(omc_status s, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

void clear_error() { g_last_error.clear(); }

bool read_file(const std::string &path, std::string &out) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out.clear();
  bool ok;
  long size = std::fseek(f, 0, SEEK_END) == 0 ? std::ftell(f) : -1;
  if (size >= 0 && std::fseek(f, 0, SEEK_SET) == 0) {  // one read of the whole file
    out.resize(static_cast<size_t>(size));
    ok = std::fread(out.data(), 1, out.size(), f) == out.size();
  } else {  // not seekable: read in blocks
    std::rewind(f);
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    ok = !std::ferror(f);
  }
  std::fclose(f);
  return ok;
}

std::vector<std::string> split_lines(const std::string &text) {
  std::vector<std::string> lines;
  size_t start = 0;
  while (start <= text.size()) {
    size_t nl = text.find('\n', start);
    if (nl == std::string::npos) {
      if (start < text.size()) lines.emplace_back(text.substr(start));
      break;
    }
    size_t end = nl;
    if (end > start && text[end - 1] == '\r') end--;
    lines.emplace_back(text.substr(start, end - start));
    start = nl + 1;
  }
  return lines;
}

std::string remove_spaces(const std::string &s) {
  std::string r;
  for (char c : s)
    if (!std::isspace(static_cast<unsigned char>(c))) r.push_back(c);
  return r;
}

bool NumberStream::next(double &v) {
  while (*p_ && std::isspace(static_cast<unsigned char>(*p_))) p_++;
  if (!*p_) return false;
  char *end = nullptr;
  v = std::strtod(p_, &end);
  if (end == p_) return false;
  p_ = end;
  return true;
}

bool NumberStream::next_int(int &v) {
  while (*p_ && std::isspace(static_cast<unsigned char>(*p_))) p_++;
  if (!*p_) return false;
  char *end = nullptr;
  long x = std::strtol(p_, &end, 10);
  if (end == p_) return false;
  v = static_cast<int>(x);
  p_ = end;
  return true;
}

}  // namespace omc

extern "C" const char *omc_last_error(void) {
  return omc::g_last_error.c_str();
}

extern "C" const char *omc_status_string(omc_status s) {
  switch (s) {
    case OMC_OK: return "ok";
    case OMC_ERR_ARG: return "invalid argument";
    case OMC_ERR_IO: return "i/o error";
    case OMC_ERR_INPUT: return "input key missing or malformed";
    case OMC_ERR_MEDIA: return "medium not found";
    case OMC_ERR_FORMAT: return "data format error";
    case OMC_ERR_NOMEM: return "out of memory";
    case OMC_ERR_CUDA: return "cuda error";
    case OMC_ERR_STACK: return "particle stack overflow";
    case OMC_ERR_LIMIT: return "device loop limit reached";
    case OMC_ERR_STATE: return "call out of order";
  }
  return "unknown status";
}
