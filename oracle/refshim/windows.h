// Minimal POSIX stand-in for the two Win32 profile-file calls that the
// reference's GradientCalc.cpp uses (GetPrivateProfileString/Int), so that its
// block split / put-back loop compiles and runs on Linux as an oracle pin.
// Test infrastructure only.
//
// Semantics kept from Win32: section and key names compare case-insensitively;
// a missing file, section or key yields the default; GetPrivateProfileInt parses
// a leading decimal integer (non-numeric text gives 0). Backslashes in the file
// name are turned into '/' (the reference opens ".\\SRRF.ini").
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cctype>
#include <string>

#define __declspec(x)

namespace refshim_detail {
inline std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}
inline bool ieq(const std::string& a, const std::string& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}
inline bool lookup(const char* sec, const char* key, const char* file, std::string* out) {
    std::string path(file);
    for (auto& c : path) if (c == '\\') c = '/';
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    std::string cur;
    bool found = false;
    while (std::fgets(line, sizeof line, f)) {
        std::string l = trim(line);
        if (l.empty() || l[0] == ';' || l[0] == '#') continue;
        if (l[0] == '[') {
            size_t e = l.find(']');
            cur = trim(l.substr(1, e == std::string::npos ? std::string::npos : e - 1));
            continue;
        }
        size_t eq = l.find('=');
        if (eq == std::string::npos) continue;
        if (ieq(cur, sec) && ieq(trim(l.substr(0, eq)), key)) {
            *out = trim(l.substr(eq + 1));
            found = true;
            break;
        }
    }
    std::fclose(f);
    return found;
}
}  // namespace refshim_detail

inline unsigned GetPrivateProfileString(const char* sec, const char* key, const char* def,
                                        char* buf, unsigned size, const char* file) {
    std::string v;
    if (!refshim_detail::lookup(sec, key, file, &v)) v = def ? def : "";
    if (size == 0) return 0;
    std::strncpy(buf, v.c_str(), size - 1);
    buf[size - 1] = 0;
    return (unsigned)std::strlen(buf);
}

inline unsigned GetPrivateProfileInt(const char* sec, const char* key, int def, const char* file) {
    std::string v;
    if (!refshim_detail::lookup(sec, key, file, &v)) return (unsigned)def;
    return (unsigned)std::atoi(v.c_str());
}
