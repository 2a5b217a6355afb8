// Mesh file reader (the microstructure read of InitMicroStruct,
// init.c:410-442): one voxel per line, "phi1 Phi phi2 i j k grain phase",
// x slowest and z fastest, the 1-based index checked against the line's
// position (init.c:420-423).
//
// The file is split at line boundaries into one chunk per thread; the chunks
// are counted, then parsed in parallel into their place.  Decimal numbers
// without an exponent and with at most 15 significant digits are converted
// as mantissa / 10^k: both operands are exact doubles, so the one division is
// correctly rounded and gives the same double as strtod (and as the
// reference's fscanf "%lf").  Every other number goes through strtod.
#include "voce_gpu.h"
#include "voce_internal.h"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                           1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// One double at p (after optional blanks); advances p.  False if none.
bool parse_double(const char *&p, const char *end, double *out)
{
    while (p < end && is_space(*p)) ++p;
    const char *s = p;
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) neg = (*p++ == '-');
    uint64_t mant = 0;
    int sig = 0, frac = 0;
    bool any = false, simple = true;
    while (p < end && *p >= '0' && *p <= '9') {
        any = true;
        if (mant || *p != '0') {
            if (sig < 19) mant = mant * 10 + (uint64_t)(*p - '0');
            ++sig;
        }
        ++p;
    }
    if (p < end && *p == '.') {
        ++p;
        while (p < end && *p >= '0' && *p <= '9') {
            any = true;
            if (mant || *p != '0') {
                if (sig < 19) mant = mant * 10 + (uint64_t)(*p - '0');
                ++sig;
            }
            ++frac;
            ++p;
        }
    }
    if (p < end && (*p == 'e' || *p == 'E' || *p == 'x' || *p == 'X' || *p == 'n' || *p == 'N' ||
                    *p == 'i' || *p == 'I'))
        simple = false;
    if (!any && simple) return false;
    if (simple && sig <= 15 && frac <= 22) {
        double v = (double)mant;
        if (frac) v /= kPow10[frac];
        *out = neg ? -v : v;
        return true;
    }
    // anything else: the C library's conversion on this token
    char buf[128];
    size_t n = 0;
    const char *q = s;
    while (q < end && !is_space(*q) && *q != '\n' && n + 1 < sizeof(buf)) buf[n++] = *q++;
    buf[n] = 0;
    char *e = nullptr;
    const double v = std::strtod(buf, &e);
    if (e == buf) return false;
    p = s + (e - buf);
    *out = v;
    return true;
}

bool parse_long(const char *&p, const char *end, long *out)
{
    while (p < end && is_space(*p)) ++p;
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) neg = (*p++ == '-');
    long v = 0;
    int nd = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        if (nd < 18) v = v * 10 + (*p - '0');
        ++nd;
        ++p;
    }
    if (!nd || nd >= 18) return false;
    *out = neg ? -v : v;
    return true;
}

inline bool blank_line(const char *p, const char *e)
{
    for (; p < e; ++p)
        if (!is_space(*p)) return false;
    return true;
}

struct Chunk {
    const char *b, *e;
    long long first = 0;   // index of its first voxel
    long long count = 0;   // voxels (non-blank lines) in it
    long long bad = -1;    // first voxel that failed, if any
    int why = 0;           // 1 short line, 2 index mismatch
};

void count_chunk(Chunk &c)
{
    long long n = 0;
    const char *p = c.b;
    while (p < c.e) {
        const char *nl = (const char *)std::memchr(p, '\n', (size_t)(c.e - p));
        const char *le = nl ? nl : c.e;
        if (!blank_line(p, le)) ++n;
        p = nl ? nl + 1 : c.e;
    }
    c.count = n;
}

void parse_chunk(Chunk &c, const int dims[3], long long nv, double *eul, int *grain, int *phase)
{
    long long v = c.first;
    const char *p = c.b;
    while (p < c.e && v < nv) {
        const char *nl = (const char *)std::memchr(p, '\n', (size_t)(c.e - p));
        const char *le = nl ? nl : c.e;
        if (blank_line(p, le)) {
            p = nl ? nl + 1 : c.e;
            continue;
        }
        double a[3];
        long iv[5];
        const char *q = p;
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k) ok = parse_double(q, le, &a[k]);
        for (int k = 0; k < 5 && ok; ++k) ok = parse_long(q, le, &iv[k]);
        if (!ok) {
            c.bad = v;
            c.why = 1;
            return;
        }
        // modulo 2^64, so that no index of up to 17 digits overflows; an
        // index whose exact linear value is v gives v
        const uint64_t idx = ((uint64_t)(iv[0] - 1) * (uint64_t)dims[1] + (uint64_t)(iv[1] - 1)) *
                                 (uint64_t)dims[2] + (uint64_t)(iv[2] - 1);
        if (idx != (uint64_t)v) {
            c.bad = v;
            c.why = 2;
            return;
        }
        eul[3 * v] = a[0];
        eul[3 * v + 1] = a[1];
        eul[3 * v + 2] = a[2];
        grain[v] = (int)iv[3];
        phase[v] = (int)iv[4];
        ++v;
        p = nl ? nl + 1 : c.e;
    }
}

}  // namespace

extern "C" int voce_mesh_read(const char *path, const int dims[3], double *eul, int *grain, int *phase)
{
    using voce::set_error;
    if (!path || !dims || !eul || !grain || !phase) return set_error(VOCE_ERR_ARG, "null argument");
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return set_error(VOCE_ERR_IO, ("cannot open mesh '" + std::string(path) + "'").c_str());
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<char> txt(sz > 0 ? (size_t)sz : 1);
    const size_t got = sz > 0 ? std::fread(txt.data(), 1, (size_t)sz, fp) : 0;
    std::fclose(fp);
    const long long nv = (long long)dims[0] * dims[1] * dims[2];
    const char *b = txt.data(), *e = b + got;
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::min<unsigned>(hw ? hw : 1, 32);
    if (got < ((size_t)1 << 20)) nt = 1;
    std::vector<Chunk> ch(nt);
    const char *cur = b;
    for (int t = 0; t < nt; ++t) {
        const char *stop = (t == nt - 1) ? e : b + (size_t)got * (t + 1) / nt;
        if (stop < cur) stop = cur;
        if (t < nt - 1) {
            const char *nl = (const char *)std::memchr(stop, '\n', (size_t)(e - stop));
            stop = nl ? nl + 1 : e;
        }
        ch[t].b = cur;
        ch[t].e = stop;
        cur = stop;
    }
    auto run = [&](auto fn) {
        if (nt == 1) {
            fn(ch[0]);
            return;
        }
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) th.emplace_back([&, t] { fn(ch[t]); });
        for (auto &x : th) x.join();
    };
    run([](Chunk &c) { count_chunk(c); });
    long long acc = 0;
    for (auto &c : ch) {
        c.first = acc;
        acc += c.count;
    }
    run([&](Chunk &c) { parse_chunk(c, dims, nv, eul, grain, phase); });
    for (const auto &c : ch)
        if (c.bad >= 0) {
            char msg[512];
            std::snprintf(msg, sizeof(msg), "mesh '%s': %s at voxel %lld", path,
                          c.why == 1 ? "short line" : "inconsistent index system", c.bad);
            return set_error(VOCE_ERR_PARSE, msg);
        }
    if (acc < nv) {
        char msg[512];
        std::snprintf(msg, sizeof(msg), "mesh '%s': short line at voxel %lld", path, acc);
        return set_error(VOCE_ERR_PARSE, msg);
    }
    return VOCE_OK;
}
