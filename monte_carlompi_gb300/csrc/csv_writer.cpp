// Per-photon CSV writer in the reference's format (monte_carlo3D.py:1621-1648):
//
//   condition wvn[um^-1] theta_n phi_n n_scat path_length[m], snow_depth[m]
//   <row: '%d %r %r %r %d %r %r'>
//
// '%r' of a float is Python's repr: the shortest digit string that reads back
// to the same value (std::to_chars gives those digits), laid out positionally
// when the decimal exponent lies in [-4, 16) and in exponent form
// ('1e-05', '1.5e+16') otherwise, with '.0' added to integral values.  FP32
// records print the shortest string that reads back to the float.  Rows are
// formatted by several threads into separate buffers and written in order.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/mcwalk.h"

namespace {

const char kHeader[] = "condition wvn[um^-1] theta_n phi_n n_scat path_length[m], snow_depth[m]\n";
// the polarised walk's file (monte_carlo3D.py:1637-1646)
const char kHeaderPol[] =
    "condition wvn[um^-1] theta_n phi_n n_scat path_length[m], snow_depth[m], Q_n, U_n, V_n\n";

// Lay out shortest digits the way Python's float repr does.
template <class T>
char *put_repr(char *p, T v) {
    if (std::isnan(v)) { memcpy(p, "nan", 3); return p + 3; }
    if (std::isinf(v)) {
        if (v < 0) *p++ = '-';
        memcpy(p, "inf", 3);
        return p + 3;
    }
    char sci[64];
    auto res = std::to_chars(sci, sci + sizeof(sci) - 1, v, std::chars_format::scientific);
    *res.ptr = '\0';
    const char *s = sci, *end = res.ptr;
    if (*s == '-') { *p++ = '-'; ++s; }
    // digits and exponent of d[.ddd]e[+-]XX
    char digits[40];
    int nd = 0;
    while (s < end && *s != 'e') {
        if (*s != '.') digits[nd++] = *s;
        ++s;
    }
    int exp10 = 0;
    if (s < end && *s == 'e') exp10 = std::atoi(s + 1);
    // to_chars writes 0 as "0e+00"
    while (nd > 1 && digits[nd - 1] == '0') --nd;
    const int decpt = exp10 + 1;  // digits d1 d2 ... with the point after decpt digits
    if (digits[0] == '0' && nd == 1) {
        memcpy(p, "0.0", 3);
        return p + 3;
    }
    if (decpt > -4 && decpt <= 16) {
        if (decpt <= 0) {
            *p++ = '0';
            *p++ = '.';
            for (int i = 0; i < -decpt; ++i) *p++ = '0';
            memcpy(p, digits, nd);
            p += nd;
        } else if (decpt >= nd) {
            memcpy(p, digits, nd);
            p += nd;
            for (int i = nd; i < decpt; ++i) *p++ = '0';
            *p++ = '.';
            *p++ = '0';
        } else {
            memcpy(p, digits, decpt);
            p += decpt;
            *p++ = '.';
            memcpy(p, digits + decpt, nd - decpt);
            p += nd - decpt;
        }
        return p;
    }
    *p++ = digits[0];
    if (nd > 1) {
        *p++ = '.';
        memcpy(p, digits + 1, nd - 1);
        p += nd - 1;
    }
    *p++ = 'e';
    int e = decpt - 1;
    *p++ = e < 0 ? '-' : '+';
    if (e < 0) e = -e;
    char eb[8];
    int ne = 0;
    do { eb[ne++] = (char)('0' + e % 10); e /= 10; } while (e);
    if (ne < 2) eb[ne++] = '0';
    while (ne) *p++ = eb[--ne];
    return p;
}

char *put_int(char *p, int64_t v) {
    auto r = std::to_chars(p, p + 24, v);
    return r.ptr;
}

constexpr size_t kMaxRow = 10 * 32 + 16;

bool mode_ok(int32_t mode) {
    return mode == MCW_MODE_F32 || mode == MCW_MODE_REPLAY64 || mode == MCW_MODE_POL64 || mode == MCW_MODE_POL32;
}

template <class R>
size_t format_rows(const R *rec, int64_t n, char *out) {
    char *p = out;
    for (int64_t i = 0; i < n; ++i) {
        const R &r = rec[i];
        p = put_int(p, r.condition);
        *p++ = ' ';
        p = put_repr(p, r.wvn);
        *p++ = ' ';
        p = put_repr(p, r.theta_n);
        *p++ = ' ';
        p = put_repr(p, r.phi_n);
        *p++ = ' ';
        p = put_int(p, r.n_scat);
        *p++ = ' ';
        p = put_repr(p, r.path_length);
        *p++ = ' ';
        p = put_repr(p, r.snow_depth);
        if constexpr (std::is_same<R, mcw_record64p>::value || std::is_same<R, mcw_record32p>::value) {
            *p++ = ' ';
            p = put_repr(p, r.stokes_q);
            *p++ = ' ';
            p = put_repr(p, r.stokes_u);
            *p++ = ' ';
            p = put_repr(p, r.stokes_v);
        }
        *p++ = '\n';
    }
    return (size_t)(p - out);
}

size_t format_any(const void *rec, int32_t mode, int64_t off, int64_t n, char *out) {
    if (mode == MCW_MODE_F32) return format_rows(static_cast<const mcw_record32 *>(rec) + off, n, out);
    if (mode == MCW_MODE_POL64) return format_rows(static_cast<const mcw_record64p *>(rec) + off, n, out);
    if (mode == MCW_MODE_POL32) return format_rows(static_cast<const mcw_record32p *>(rec) + off, n, out);
    return format_rows(static_cast<const mcw_record64 *>(rec) + off, n, out);
}

const char *header_of(int32_t mode) {
    return (mode == MCW_MODE_POL64 || mode == MCW_MODE_POL32) ? kHeaderPol : kHeader;
}

}  // namespace

extern "C" {

int mcw_format_csv(const void *records, int32_t mode, int64_t n, int32_t header, char *buf, size_t cap,
                   size_t *used) {
    if ((!records && n > 0) || n < 0 || !used) return MCW_ERR_ARG;
    if (!mode_ok(mode)) return MCW_ERR_ARG;
    const char *hdr = header_of(mode);
    const size_t hlen = strlen(hdr);
    std::string tmp;
    tmp.resize((size_t)n * kMaxRow + hlen + 1);
    size_t len = 0;
    if (header) {
        memcpy(&tmp[0], hdr, hlen);
        len = hlen;
    }
    len += format_any(records, mode, 0, n, &tmp[len]);
    *used = len;
    if (buf && cap >= len) memcpy(buf, tmp.data(), len);
    return (buf && cap < len) ? MCW_ERR_ARG : MCW_OK;
}

int mcw_write_csv(const char *path, const void *records, int32_t mode, int64_t n, int32_t n_threads) {
    if (!path || (!records && n > 0) || n < 0) return MCW_ERR_ARG;
    if (!mode_ok(mode)) return MCW_ERR_ARG;
    if (n_threads <= 0) n_threads = (int32_t)std::max(1u, std::thread::hardware_concurrency());
    FILE *f = fopen(path, "wb");
    if (!f) return MCW_ERR_ARG;
    int rc = MCW_OK;
    const char *hdr = header_of(mode);
    const size_t hlen = strlen(hdr);
    if (fwrite(hdr, 1, hlen, f) != hlen) rc = MCW_ERR_ARG;
    // chunks of rows formatted by n_threads workers, written in order
    const int64_t chunk = 1 << 16;
    std::vector<std::string> bufs(n_threads);
    std::vector<size_t> lens(n_threads);
    for (int64_t base = 0; rc == MCW_OK && base < n; base += chunk * n_threads) {
        std::vector<std::thread> th;
        for (int t = 0; t < n_threads; ++t) {
            const int64_t lo = base + t * chunk;
            const int64_t cnt = std::max<int64_t>(0, std::min<int64_t>(chunk, n - lo));
            lens[t] = 0;
            if (cnt == 0) continue;
            bufs[t].resize((size_t)cnt * kMaxRow);
            th.emplace_back([&, t, lo, cnt] { lens[t] = format_any(records, mode, lo, cnt, &bufs[t][0]); });
        }
        for (auto &x : th) x.join();
        for (int t = 0; t < n_threads; ++t)
            if (lens[t] && fwrite(bufs[t].data(), 1, lens[t], f) != lens[t]) rc = MCW_ERR_ARG;
    }
    if (fclose(f) != 0) rc = MCW_ERR_ARG;
    return rc;
}

}  // extern "C"
