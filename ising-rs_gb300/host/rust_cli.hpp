// rust_cli.hpp — the reference's command-line conventions, restated in C++ for
// the drop-in drivers (gpu_fss, fss).
//
// Mirrors src/cli.rs of faulknco/ising-rs:
//   get_arg            cli.rs:10-16   "Error: {flag} requires a value", exit 1
//   parse_arg          cli.rs:19-28   "Error: invalid value '{v}' for {flag}: {e}"
//                                     with Rust's FromStr error texts
//   check_help         cli.rs:46-51   usage on stderr, exit 0
//   warn_unknown_flags cli.rs:54-68   "Warning: unknown flag '{arg}' (ignored)"
// plus Rust's f64 Display (shortest round-trip digits, no exponent) for the
// messages that print a float, and `.expect()` panics (exit code 101).
#pragma once

#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

namespace rcli {

[[noreturn]] inline void die(const std::string& msg) {
    fprintf(stderr, "%s\n", msg.c_str());
    exit(1);
}

// Rust's `expect` on an Err: panic message naming the source file, exit 101.
[[noreturn]] inline void panic_expect(const char* src, const char* what, const std::string& err) {
    fprintf(stderr, "thread 'main' panicked at %s:\n%s: %s\n", src, what, err.c_str());
    exit(101);
}

// f64 Display as Rust prints it: shortest round-trip digits, no exponent.
inline std::string rust_f64(double x) {
    if (isnan(x)) return "NaN";
    if (isinf(x)) return x < 0 ? "-inf" : "inf";
    if (x == 0.0) return signbit(x) ? "-0" : "0";
    char buf[64];
    int p = 1;
    for (; p <= 17; ++p) {
        snprintf(buf, sizeof buf, "%.*e", p - 1, x);
        if (strtod(buf, nullptr) == x) break;
    }
    std::string s(buf);
    bool neg = s[0] == '-';
    if (neg) s = s.substr(1);
    size_t epos = s.find('e');
    int exp10 = atoi(s.c_str() + epos + 1);
    std::string digits;
    for (size_t i = 0; i < epos; ++i)
        if (s[i] != '.') digits += s[i];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    std::string out;
    if (exp10 >= 0) {
        if ((int)digits.size() <= exp10 + 1) {
            out = digits + std::string(exp10 + 1 - digits.size(), '0');
        } else {
            out = digits.substr(0, exp10 + 1) + "." + digits.substr(exp10 + 1);
        }
    } else {
        out = "0." + std::string(-exp10 - 1, '0') + digits;
    }
    return (neg ? "-" : "") + out;
}

inline std::string get_arg(int argc, char** argv, int i, const char* flag) {
    if (i + 1 >= argc) die(std::string("Error: ") + flag + " requires a value");
    return argv[i + 1];
}

// Rust's str::parse::<usize>/<u64>: optional '+', decimal digits only.
inline bool parse_unsigned(const std::string& v, uint64_t* out, std::string* err) {
    if (v.empty()) {
        *err = "cannot parse integer from empty string";
        return false;
    }
    size_t i = 0;
    if (v[0] == '+') i = 1;
    if (i >= v.size()) {
        *err = "invalid digit found in string";
        return false;
    }
    uint64_t x = 0;
    for (; i < v.size(); ++i) {
        if (v[i] < '0' || v[i] > '9') {
            *err = "invalid digit found in string";
            return false;
        }
        uint64_t d = (uint64_t)(v[i] - '0');
        if (x > (UINT64_MAX - d) / 10) {
            *err = "number too large to fit in target type";
            return false;
        }
        x = x * 10 + d;
    }
    *out = x;
    return true;
}

inline bool parse_f64(const std::string& v, double* out, std::string* err) {
    if (v.empty()) {
        *err = "cannot parse float from empty string";
        return false;
    }
    for (char c : v)
        if (isspace((unsigned char)c) || c == 'x' || c == 'X' || c == 'p' || c == 'P') {
            *err = "invalid float literal";
            return false;
        }
    char* end = nullptr;
    errno = 0;
    double x = strtod(v.c_str(), &end);
    if (end == v.c_str() || *end != '\0') {
        *err = "invalid float literal";
        return false;
    }
    *out = x;
    return true;
}

template <class T>
T parse_arg(int argc, char** argv, int i, const char* flag);

template <>
inline uint64_t parse_arg<uint64_t>(int argc, char** argv, int i, const char* flag) {
    std::string v = get_arg(argc, argv, i, flag), err;
    uint64_t x = 0;
    if (!parse_unsigned(v, &x, &err))
        die("Error: invalid value '" + v + "' for " + flag + ": " + err);
    return x;
}

template <>
inline double parse_arg<double>(int argc, char** argv, int i, const char* flag) {
    std::string v = get_arg(argc, argv, i, flag), err;
    double x = 0;
    if (!parse_f64(v, &x, &err)) die("Error: invalid value '" + v + "' for " + flag + ": " + err);
    return x;
}

// Comma-separated sizes, each trimmed; entries that do not parse as usize are
// dropped (`.split(',').filter_map(|s| s.trim().parse().ok())`).
inline std::vector<int> parse_sizes(const std::string& list, bool trim) {
    std::vector<int> out;
    size_t p = 0;
    while (p <= list.size()) {
        size_t q = list.find(',', p);
        if (q == std::string::npos) q = list.size();
        std::string tok = list.substr(p, q - p);
        if (trim) {
            size_t b = tok.find_first_not_of(" \t\n\r"), e = tok.find_last_not_of(" \t\n\r");
            tok = b == std::string::npos ? "" : tok.substr(b, e - b + 1);
        }
        uint64_t v = 0;
        std::string err;
        if (parse_unsigned(tok, &v, &err) && v <= 0x7FFFFFFF) out.push_back((int)v);
        p = q + 1;
    }
    return out;
}

inline void check_help(int argc, char** argv, const char* usage) {
    for (int i = 1; i < argc; ++i)
        if (!strcmp(argv[i], "--help") || !strcmp(argv[i], "-h")) {
            fprintf(stderr, "%s\n", usage);
            exit(0);
        }
}

inline void warn_unknown_flags(int argc, char** argv, const std::vector<std::string>& known) {
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--", 0) != 0) continue;
        bool found = false;
        for (const auto& k : known) found = found || k == a;
        if (found) ++i;  // skip its value (flags without one skip their successor too)
        else fprintf(stderr, "Warning: unknown flag '%s' (ignored)\n", a.c_str());
    }
}

inline std::string join_path(const std::string& dir, const std::string& name) {
    if (dir.empty()) return name;
    if (dir.back() == '/') return dir + name;
    return dir + "/" + name;
}

// fs::create_dir_all; on failure *err holds Rust's io::Error Debug text.
inline bool mkdirs(const std::string& path, std::string* err) {
    std::string cur;
    size_t i = 0;
    if (!path.empty() && path[0] == '/') cur = "/", i = 1;
    while (i <= path.size()) {
        size_t j = path.find('/', i);
        if (j == std::string::npos) j = path.size();
        if (j > i) {
            cur += path.substr(i, j - i);
            if (mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) {
                *err = std::string("Os { code: ") + std::to_string(errno) + ", message: \"" +
                       strerror(errno) + "\" }";
                return false;
            }
            struct stat st;
            if (stat(cur.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) {
                *err = "Os { code: 17, message: \"File exists\" }";
                return false;
            }
            cur += "/";
        }
        i = j + 1;
    }
    return true;
}

}  // namespace rcli
