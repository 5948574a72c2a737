// Minimal stand-in for the subset of glog the reference uses
// (include/log.hpp:31-38, LOG(sev) and CHECK(cond) << msg at its call sites).
// Written from those call sites only; messages go to stderr and a failed
// CHECK aborts, as glog's does.  Test infrastructure for building the
// reference baseline; not part of the engine.
#pragma once
// The real header pulls these in; the reference relies on them transitively.
#include <errno.h>
#include <time.h>
#include <unistd.h>

#include <cstdlib>
#include <iostream>
#include <ostream>
#include <sstream>
#include <string>
#include <vector>

namespace google {
enum LogSeverity { INFO = 0, WARNING = 1, ERROR = 2, FATAL = 3 };
struct LogMessage {
    static const int kMaxLogMessageLen = 30000;
};
inline void InitGoogleLogging(const char *) {}
}  // namespace google

static int FLAGS_minloglevel = google::WARNING;
static bool FLAGS_logtostderr = true;
static bool FLAGS_log_prefix = false;

namespace ptw_glog_shim {
struct Line {
    std::ostringstream os;
    int sev;
    explicit Line(int s) : sev(s) {}
    ~Line()
    {
        if (sev >= FLAGS_minloglevel || sev == google::FATAL) std::cerr << os.str() << std::endl;
        if (sev == google::FATAL) std::abort();
    }
    template <typename T> Line &operator<<(const T &x)
    {
        os << x;
        return *this;
    }
    Line &operator<<(const char *s)  // also takes variable-length char arrays
    {
        os << s;
        return *this;
    }
};
struct Voidify {
    void operator&(Line &) {}
};
}  // namespace ptw_glog_shim

#define LOG(sev) ptw_glog_shim::Line(google::sev)
#define CHECK(cond)                                                                       \
    (cond) ? (void)0                                                                      \
           : ptw_glog_shim::Voidify() &                                                   \
                 ptw_glog_shim::Line(google::FATAL) << "Check failed: " #cond " (" << __FILE__ \
                                                    << ":" << __LINE__ << ") "
