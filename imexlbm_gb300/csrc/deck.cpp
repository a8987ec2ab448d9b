// Input deck parsing: imex_deck_parse / imex_deck_read.
//
// The reference reads nine numbers with std::istream >> into
// rho0 R Re / u0 Time inter / sx sy sz (src/System.cpp:22-24), where Re,
// Time, inter, sx, sy and sz are ints (src/System.hpp:16-18), then derives
// Ma, miu and tau left to right as written (src/System.cpp:26-28).  This
// parser uses the same extraction (an int field stops at the first
// non-digit character) and the same derivations.  Where the reference would
// abort on a missing file or continue with zeroed fields after a failed
// extraction, this returns IMEX_ERR_DECK with a message.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"

namespace {

const char* skip_space(const char* s)
{
    while (*s && std::isspace(static_cast<unsigned char>(*s))) ++s;
    return s;
}

bool extract_int(const char*& s, int& out)
{
    const char* p = skip_space(s);
    const char* b = p;
    if (*p == '+' || *p == '-') ++p;
    if (!std::isdigit(static_cast<unsigned char>(*p))) return false;
    while (std::isdigit(static_cast<unsigned char>(*p))) ++p;
    const std::string tok(b, p);
    const long v = std::strtol(tok.c_str(), nullptr, 10);
    if (v > 2147483647L || v < -2147483647L - 1) return false;
    out = static_cast<int>(v);
    s = p;
    return true;
}

bool extract_double(const char*& s, double& out)
{
    const char* p = skip_space(s);
    const char* b = p;
    int digits = 0;
    if (*p == '+' || *p == '-') ++p;
    while (std::isdigit(static_cast<unsigned char>(*p))) ++p, ++digits;
    if (*p == '.') {
        ++p;
        while (std::isdigit(static_cast<unsigned char>(*p))) ++p, ++digits;
    }
    if (!digits) return false;
    if (*p == 'e' || *p == 'E') {
        const char* t = p + 1;
        if (*t == '+' || *t == '-') ++t;
        if (std::isdigit(static_cast<unsigned char>(*t))) {
            while (std::isdigit(static_cast<unsigned char>(*t))) ++t;
            p = t;
        }
    }
    const std::string tok(b, p);
    out = std::strtod(tok.c_str(), nullptr);
    s = p;
    return true;
}

}  // namespace

extern "C" int imex_deck_parse(const char* text, imex_deck* d)
{
    if (!text || !d) return imex::set_thread_error(IMEX_ERR_ARG, "imex_deck_parse: null argument");
    imex_deck r;
    std::memset(&r, 0, sizeof r);
    const char* s = text;
    static const char* names[9] = {"rho0", "R", "Re", "u0", "Time", "inter", "sx", "sy", "sz"};
    int field = 0;
    bool ok = extract_double(s, r.rho0) && ++field && extract_double(s, r.R) && ++field && extract_int(s, r.Re) &&
              ++field && extract_double(s, r.u0) && ++field && extract_int(s, r.Time) && ++field &&
              extract_int(s, r.inter) && ++field && extract_int(s, r.sx) && ++field && extract_int(s, r.sy) &&
              ++field && extract_int(s, r.sz) && ++field;
    if (!ok) return imex::set_thread_error(IMEX_ERR_DECK, std::string("deck: cannot read field ") + names[field]);
    r.cs2 = 1.0 / 3.0;
    r.cs = std::sqrt(r.cs2);
    r.Ma = r.u0 / r.cs;
    r.miu = r.rho0 * r.u0 * r.sx / 2.0 / 3.1415926 / r.Re;
    r.tau = r.u0 * r.sx / r.Re / r.cs2 / 2.0 / 3.1415926;
    *d = r;
    return IMEX_OK;
}

extern "C" int imex_deck_read(const char* path, imex_deck* d)
{
    if (!path || !d) return imex::set_thread_error(IMEX_ERR_ARG, "imex_deck_read: null argument");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return imex::set_thread_error(IMEX_ERR_DECK, std::string("FATAL: cannot open ") + path);
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, n);
    std::fclose(fp);
    return imex_deck_parse(text.c_str(), d);
}
