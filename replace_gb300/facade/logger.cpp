#include "logger.h"

#include <cstdio>
#include <cstdlib>

namespace replace {

Logger::Logger(std::string name, int verbose) : verbose_(verbose), name_(std::move(name)) {}

void Logger::proc(std::string s, int v) {
  if (!quiet(v)) printf("[PROC] %s\n", s.c_str());
}
void Logger::procBegin(std::string s, int v) {
  if (!quiet(v)) printf("[PROC] Begin %s ...\n", s.c_str());
}
void Logger::procEnd(std::string s, int v) {
  if (!quiet(v)) printf("[PROC] End %s\n", s.c_str());
}

void Logger::error(std::string s, int code, int) {
  // printed whatever the level: the process ends here
  printf("[ERROR] %s (%s-%d)\n", s.c_str(), name_.c_str(), code);
  fflush(stdout);
  exit(code);
}

void Logger::warn(std::string s, int code, int v) {
  if (!quiet(v)) printf("[WARN] %s (%s-%d)\n", s.c_str(), name_.c_str(), code);
}

void Logger::infoInt(std::string s, int val, int v) {
  if (!quiet(v)) printf("[INFO] %s = %d\n", s.c_str(), val);
}
void Logger::infoIntPair(std::string s, int a, int b, int v) {
  if (!quiet(v)) printf("[INFO] %s = (%d, %d)\n", s.c_str(), a, b);
}
void Logger::infoInt64(std::string s, int64_t val, int v) {
  if (!quiet(v)) printf("[INFO] %s = %lld\n", s.c_str(), (long long)val);
}
void Logger::infoFloat(std::string s, float val, int v) {
  if (!quiet(v)) printf("[INFO] %s = %.6f\n", s.c_str(), val);
}
void Logger::infoFloatSignificant(std::string s, float val, int v) {
  if (!quiet(v)) printf("[INFO] %s = %g\n", s.c_str(), val);
}
void Logger::infoFloatPair(std::string s, float a, float b, int v) {
  if (!quiet(v)) printf("[INFO] %s = (%.6f, %.6f)\n", s.c_str(), a, b);
}
void Logger::infoString(std::string s, int v) {
  if (!quiet(v)) printf("[INFO] %s\n", s.c_str());
}
void Logger::infoString(std::string s, std::string val, int v) {
  if (!quiet(v)) printf("[INFO] %s = %s\n", s.c_str(), val.c_str());
}
void Logger::infoRuntime(std::string s, double t, int v) {
  if (!quiet(v)) printf("[INFO] %sRuntime = %.4f\n", s.c_str(), t);
}

}  // namespace replace
