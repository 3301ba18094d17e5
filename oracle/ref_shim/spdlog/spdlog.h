// Minimal stand-in for spdlog used when compiling the reference sources.
//
// TEST INFRASTRUCTURE ONLY. Messages are formatted by replacing each "{}" with the next
// argument and kept in a small in-process log so the harness can read the reference's
// own stage-timing lines ("StatMC denoise completed in N ms"). They are printed to stderr
// only when the environment variable RPD_REF_LOG is set.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

namespace spdlog {
namespace shim {

inline std::vector<std::string>& log_lines() {
    static std::vector<std::string> lines;
    return lines;
}

inline void append_arg(std::ostringstream&, const char*& fmt) {
    while (*fmt) {
        if (fmt[0] == '{' && fmt[1] == '}') return;
        ++fmt;
    }
}

inline void format_into(std::ostringstream& out, const char* fmt) { out << fmt; }

template <typename A, typename... Rest>
inline void format_into(std::ostringstream& out, const char* fmt, const A& a, const Rest&... rest) {
    while (*fmt) {
        if (fmt[0] == '{' && fmt[1] == '}') {
            out << a;
            format_into(out, fmt + 2, rest...);
            return;
        }
        out << *fmt++;
    }
}

template <typename... Args>
inline void emit(const char* level, const char* fmt, const Args&... args) {
    std::ostringstream out;
    format_into(out, fmt, args...);
    #ifdef _OPENMP
    #pragma omp critical(rpd_shim_log)
    #endif
    {
        auto& lines = log_lines();
        if (lines.size() > 4096) lines.erase(lines.begin(), lines.begin() + 2048);
        lines.push_back(out.str());
    }
    if (std::getenv("RPD_REF_LOG")) std::fprintf(stderr, "[%s] %s\n", level, out.str().c_str());
}

}  // namespace shim

template <typename... Args>
inline void info(const char* fmt, const Args&... args) { shim::emit("info", fmt, args...); }
template <typename... Args>
inline void warn(const char* fmt, const Args&... args) { shim::emit("warn", fmt, args...); }
template <typename... Args>
inline void error(const char* fmt, const Args&... args) { shim::emit("error", fmt, args...); }

}  // namespace spdlog
