// Number parsing and formatting shared by the sample reader and the event
// averager: the same values as strtod / printf, faster.
#pragma once

#include <algorithm>
#include <charconv>
#include <cstdlib>
#include <cstring>

namespace hbt {

inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// parse_numbers on the span [b, e) (not NUL-terminated).  std::from_chars
// and strtod are both correctly rounded, so a token both accept gives the
// same double; any token from_chars does not take whole (a leading '+', hex,
// overflow, trailing junk) is handed to strtod on a NUL-terminated copy, and
// parsing resumes where strtod stopped, exactly as the strtod loop would.
inline int parse_span(const char *b, const char *e, double *out, int count) {
    int k = 0;
    const char *s = b;
    char tok[128];
    while (k < count) {
        while (s < e && is_space(*s)) s++;
        if (s >= e) break;
        double v = 0.0;
        const std::from_chars_result r = std::from_chars(s, e, v);
        if (r.ec == std::errc() && *s != '+' && (r.ptr == e || is_space(*r.ptr))) {
            out[k++] = v;
            s = r.ptr;
            continue;
        }
        const char *t = s;
        while (t < e && !is_space(*t)) t++;
        const size_t n = std::min<size_t>(t - s, sizeof(tok) - 1);
        memcpy(tok, s, n);
        tok[n] = '\0';
        char *end = nullptr;
        v = strtod(tok, &end);
        if (end == tok) break;
        out[k++] = v;
        s += end - tok;
    }
    return k;
}

// printf("%.<prec>e") of v into p (no padding); returns the end.
inline char *put_sci(char *p, double v, int prec) {
    const std::to_chars_result r = std::to_chars(p, p + 48, v, std::chars_format::scientific, prec);
    return r.ptr;
}

}  // namespace hbt
