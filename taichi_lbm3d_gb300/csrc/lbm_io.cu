// Host-side reader of the reference's ASCII fields: the geometry, psi and
// grey-scale files that init_geo loads with np.loadtxt (x fastest,
// Single_phase/LBM_3D_SinglePhase_Solver.py:173-177, 2phase/lbm_solver_3d_2phase_sparse.py:195-203,
// Grey_Scale/lbm_solver_3d_Macro_Sukop.py init_geo).  A 256^3 file is 16.8 M numbers;
// the file is read once, cut into one chunk per host thread at whitespace, and
// each chunk is counted and then parsed in place.  Single-digit tokens (the 0/1
// solid flags) take a direct path; every other token goes through
// std::from_chars, which rounds correctly, so values equal np.loadtxt's.
#include <algorithm>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "lbm_internal.h"

namespace {

inline bool io_space(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

int64_t io_count(const char* p, const char* e) {
    int64_t n = 0;
    while (p < e) {
        while (p < e && io_space(*p)) ++p;
        if (p == e) break;
        ++n;
        while (p < e && !io_space(*p)) ++p;
    }
    return n;
}

// Parses the tokens of [p, e) into out; returns the offset of the first bad
// token from p, or -1.
int64_t io_parse(const char* p, const char* e, double* out) {
    const char* b = p;
    while (p < e) {
        while (p < e && io_space(*p)) ++p;
        if (p == e) break;
        const char* t = p;
        while (p < e && !io_space(*p)) ++p;
        if (p - t == 1 && *t >= '0' && *t <= '9') {
            *out++ = (double)(*t - '0');
            continue;
        }
        const char* s = (*t == '+' && p - t > 1) ? t + 1 : t;
        double v = 0.0;
        const std::from_chars_result r = std::from_chars(s, p, v);
        if (r.ec != std::errc() || r.ptr != p) return (int64_t)(t - b);
        *out++ = v;
    }
    return -1;
}

}  // namespace

extern "C" int lbm_read_ascii(const char* path, double* out, int64_t n, int64_t* count) {
    if (!path || !count) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_read_ascii: NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return lbm_set_err(nullptr, LBM_EINVAL, std::string("lbm_read_ascii: cannot open ") + path);
    std::vector<char> buf;
    bool failed = std::fseek(f, 0, SEEK_END) != 0;
    const long size = failed ? -1 : std::ftell(f);
    if (size >= 0 && std::fseek(f, 0, SEEK_SET) == 0) {
        buf.resize((size_t)size);
        failed = std::fread(buf.data(), 1, buf.size(), f) != buf.size();
    } else {
        failed = true;
    }
    failed = failed || std::ferror(f) != 0;
    std::fclose(f);
    if (failed) return lbm_set_err(nullptr, LBM_EINVAL, std::string("lbm_read_ascii: read error on ") + path);

    // chunk boundaries at whitespace, one chunk per thread
    const char* base = buf.data();
    const char* end = base + buf.size();
    const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const int nt = buf.size() < ((size_t)1 << 20) ? 1 : (int)hw;
    std::vector<const char*> cut(nt + 1);
    cut[0] = base;
    cut[nt] = end;
    for (int t = 1; t < nt; ++t) {
        const char* c = base + buf.size() * t / nt;
        if (c < cut[t - 1]) c = cut[t - 1];
        while (c < end && !io_space(*c)) ++c;
        cut[t] = c;
    }
    std::vector<int64_t> cnt(nt, 0);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) th.emplace_back([&, t] { cnt[t] = io_count(cut[t], cut[t + 1]); });
        for (auto& x : th) x.join();
    }
    int64_t total = 0;
    std::vector<int64_t> off(nt, 0);
    for (int t = 0; t < nt; ++t) {
        off[t] = total;
        total += cnt[t];
    }
    *count = total;
    if (!out) return LBM_OK;
    if (total != n)
        return lbm_set_err(nullptr, LBM_EINVAL, std::string("lbm_read_ascii: ") + path + " holds " + std::to_string(total) +
                                                    " values, expected " + std::to_string(n));
    std::vector<int64_t> bad(nt, -1);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&, t] { bad[t] = io_parse(cut[t], cut[t + 1], out + off[t]); });
        for (auto& x : th) x.join();
    }
    for (int t = 0; t < nt; ++t) {
        if (bad[t] >= 0) {
            const int64_t at = (int64_t)(cut[t] - base) + bad[t];
            std::string tok;
            for (const char* q = base + at; q < end && !io_space(*q) && tok.size() < 40; ++q) tok += *q;
            return lbm_set_err(nullptr, LBM_EINVAL, std::string("lbm_read_ascii: not a number at byte ") +
                                                        std::to_string(at) + " of " + path + ": '" + tok + "'");
        }
    }
    return LBM_OK;
}
