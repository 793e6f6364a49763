// Minimal logging shim used ONLY to compile nla3d's own sources into the
// oracle build (oracle/_ref).  The logging library the reference vendors as a
// git submodule is empty in this checkout, so this header provides the subset
// of its macro/type surface that nla3d's hot-path sources call (sys.h:65-88,
// FEStorage.cpp:30, SparseMatrix.cpp:84, isoparametric.cpp:177, ...).
//
// Behaviour:
//   * LOG(INFO/WARNING/ERROR/DEBUG) -> discarded unless NLA3D_SHIM_VERBOSE is set.
//   * LOG(FATAL) / failed CHECK     -> throws nla3d_shim::FatalError, so the
//                                      harness can turn an abort of the
//                                      reference into an error status.
//   * TIMED_SCOPE(obj, "name")      -> a steady_clock scope timer whose total
//                                      per name is readable through
//                                      nla3d_shim::timers().
// This is test infrastructure, written from the reference's call sites; it is
// not a copy of the third-party library.
#pragma once

// Standard headers that nla3d's sources rely on receiving transitively
// through the logging header (e.g. std::shared_ptr in SparseMatrix.h:129).
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <functional>
#include <memory>
#include <unordered_map>
#include <utility>
#include <vector>
#include <chrono>
#include <exception>
#include <cstdlib>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

namespace nla3d_shim {

struct FatalError : public std::runtime_error {
  explicit FatalError(const std::string& m) : std::runtime_error(m) {}
};

inline std::map<std::string, double>& timers() {
  static std::map<std::string, double> t;
  return t;
}

inline bool verbose() {
  static int v = std::getenv("NLA3D_SHIM_VERBOSE") ? 1 : 0;
  return v != 0;
}

enum class Sev { Trace, Debug, Info, Warning, Error, Fatal, Verbose };

class LogLine {
 public:
  explicit LogLine(Sev s, bool on = true) : sev_(s), on_(on) {}
  LogLine(const LogLine&) = delete;
  ~LogLine() noexcept(false) {
    if (!on_) return;
    if (sev_ == Sev::Fatal && !std::uncaught_exception()) throw FatalError(ss_.str());
    if (verbose()) std::cerr << "[nla3d] " << ss_.str() << std::endl;
  }
  template <class T>
  LogLine& operator<<(const T& v) {
    if (on_) ss_ << v;
    return *this;
  }
  LogLine& operator<<(std::ostream& (*f)(std::ostream&)) {
    if (on_) ss_ << f;
    return *this;
  }
  std::ostream& stream() { return ss_; }

 private:
  Sev sev_;
  bool on_;
  std::ostringstream ss_;
};

class ScopeTimer {
 public:
  explicit ScopeTimer(const char* name)
      : name_(name), t0_(std::chrono::steady_clock::now()) {}
  ~ScopeTimer() {
    auto t1 = std::chrono::steady_clock::now();
    timers()[name_] += std::chrono::duration<double>(t1 - t0_).count();
  }
  void checkpoint(const char*) {}

 private:
  std::string name_;
  std::chrono::steady_clock::time_point t0_;
};

}  // namespace nla3d_shim

#define NLA3D_SHIM_SEV_INFO nla3d_shim::Sev::Info
#define NLA3D_SHIM_SEV_WARNING nla3d_shim::Sev::Warning
#define NLA3D_SHIM_SEV_ERROR nla3d_shim::Sev::Error
#define NLA3D_SHIM_SEV_FATAL nla3d_shim::Sev::Fatal
#define NLA3D_SHIM_SEV_DEBUG nla3d_shim::Sev::Debug
#define NLA3D_SHIM_SEV_TRACE nla3d_shim::Sev::Trace

#define LOG(sev) nla3d_shim::LogLine(NLA3D_SHIM_SEV_##sev)
#define DLOG(sev) nla3d_shim::LogLine(NLA3D_SHIM_SEV_##sev, false)
#define LOG_IF(cond, sev) nla3d_shim::LogLine(NLA3D_SHIM_SEV_##sev, (cond))
#define LOG_N_TIMES(n, sev) nla3d_shim::LogLine(NLA3D_SHIM_SEV_##sev, false)
#define CHECK(cond) \
  nla3d_shim::LogLine(nla3d_shim::Sev::Fatal, !(cond)) << "CHECK failed: " #cond " "
#define CHECK_EQ(a, b) CHECK((a) == (b))
#define CHECK_NE(a, b) CHECK((a) != (b))
#define CHECK_LT(a, b) CHECK((a) < (b))
#define CHECK_GT(a, b) CHECK((a) > (b))
#define CHECK_LE(a, b) CHECK((a) <= (b))
#define CHECK_GE(a, b) CHECK((a) >= (b))
#define CHECK_NOTNULL(x) (x)
#define DCHECK(cond) DLOG(INFO)
#define TIMED_SCOPE(obj, name) nla3d_shim::ScopeTimer obj(name)
#define TIMED_BLOCK(obj, name) for (nla3d_shim::ScopeTimer obj(name), *obj##_once = &obj; obj##_once; obj##_once = nullptr)
#define INITIALIZE_EASYLOGGINGPP
#define MAKE_LOGGABLE(ClassType, ClassInstance, OutputStreamInstance) \
  std::ostream& operator<<(std::ostream& OutputStreamInstance, const ClassType& ClassInstance)

// The configuration surface touched by nla3d's LogInitializer (sys.h:65-88).
namespace el {
enum class Level { Global, Trace, Debug, Fatal, Error, Warning, Verbose, Info };
enum class ConfigurationType {
  Enabled, ToFile, ToStandardOutput, Format, Filename, SubsecondPrecision,
  MillisecondsWidth, PerformanceTracking, MaxLogFileSize, LogFlushThreshold
};
enum class LoggingFlag { ColoredTerminalOutput };
class Configurations {
 public:
  void setToDefault() {}
  void setGlobally(ConfigurationType, const std::string&) {}
  void set(Level, ConfigurationType, const std::string&) {}
};
class Loggers {
 public:
  static void reconfigureAllLoggers(const Configurations&) {}
  static void addFlag(LoggingFlag) {}
};
}  // namespace el
