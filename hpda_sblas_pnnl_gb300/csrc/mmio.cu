// MatrixMarket reading (host code only): the NIST mmio entry points the
// reference's test programs call (the reference vendors them header-only in its
// include/mmio.h: declarations and bodies) and a multi-threaded reader of
// a whole coordinate file, the replacement of those programs' per-entry fscanf
// loop (test/dspmv_test_dgx1.cu:133-181).
//
// The whole-file reader maps the file, splits its data section into one
// byte range per thread at line starts, and makes three passes:
//   1. every thread counts its entry lines;
//   2. with the exclusive prefix of those counts as its first entry index,
//      every thread parses its lines straight into the output arrays (only
//      entries below the announced nnz) and counts its off-diagonals;
//   3. (symmetric expansion only) every thread appends the mirrors of its
//      own stored entries at the prefix of the off-diagonal counts, read
//      back from the output arrays.
// Results do not depend on the number of threads.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mmio.h"
#include "sblas_internal.h"

namespace sblas {
namespace {

inline bool is_space(char c)
{
    return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f';
}

// Next whitespace-separated token of [p, e) copied into buf (NUL-ended);
// false when the line holds no further token or the token is too long.
bool next_token(const char *&p, const char *e, char *buf, size_t cap)
{
    while (p < e && is_space(*p)) ++p;
    if (p >= e) return false;
    size_t k = 0;
    while (p < e && !is_space(*p)) {
        if (k + 1 >= cap) return false;
        buf[k++] = *p++;
    }
    buf[k] = '\0';
    return true;
}

// Decimal integer token (optional sign) as strtoll reads it, whole token.
bool parse_ll(const char *tok, long long *v)
{
    errno = 0;
    char *end = nullptr;
    const long long r = std::strtoll(tok, &end, 10);
    if (end == tok || *end != '\0' || errno == ERANGE) return false;
    *v = r;
    return true;
}

// The next token of [p, e) read in place as a decimal integer, accepting
// what strtoll (base 10) accepts as a whole token: an optional sign, then
// one or more digits and nothing else up to the next whitespace; false on
// any other character, no digits, or a value outside long long.  Indices
// and integer values take this path (no copy, no errno, no locale); it was
// a copy plus strtoll per token, the largest cost of parsing a line.
bool scan_ll(const char *&p, const char *e, long long *v)
{
    while (p < e && is_space(*p)) ++p;
    if (p >= e) return false;
    const bool neg = (*p == '-');
    if (*p == '+' || *p == '-') ++p;
    const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
    const char *d0 = p;
    unsigned long long acc = 0;
    bool over = false;
    for (; p < e && *p >= '0' && *p <= '9'; ++p) {
        const unsigned dig = (unsigned)(*p - '0');
        if (acc > (lim - dig) / 10) over = true;
        else acc = acc * 10 + dig;
    }
    if (p == d0 || over || (p < e && !is_space(*p))) return false;
    *v = neg ? (long long)(0ull - acc) : (long long)acc;
    return true;
}

// The decimal number [p, e) (one whole token) by Clinger's fast path (W. D.
// Clinger, "How to Read Floating Point Numbers Accurately", PLDI 1990): the
// token is W * 10^E with a decimal significand W <= 2^53 and |E| <= 22, so
// W and 10^|E| are both exact doubles and one IEEE multiplication (E >= 0)
// or division (E < 0) rounds once, to the double strtod returns.  Accepts
// [sign] digits [. digits] [e|E [sign] digits] with at least one significand
// digit; false for any other token (inf, nan, hexadecimal, 17 or more
// significant digits -- W >= 10^16 > 2^53 --, W > 2^53, |E| > 22, other
// characters): the caller then converts it with strtod.
bool fast_double(const char *p, const char *e, double *v)
{
    static const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,
                                      1e8,  1e9,  1e10, 1e11, 1e12, 1e13, 1e14, 1e15,
                                      1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = (*p++ == '-');
    unsigned long long w = 0;
    int sig = 0, ndig = 0, scale = 0;
    for (; p < e && *p >= '0' && *p <= '9'; ++p, ++ndig) {
        if (w == 0 && *p == '0') continue;            // leading zeros
        if (++sig > 16) return false;
        w = w * 10 + (unsigned)(*p - '0');
    }
    if (p < e && *p == '.') {
        for (++p; p < e && *p >= '0' && *p <= '9'; ++p, ++ndig) {
            --scale;
            if (w == 0 && *p == '0') continue;
            if (++sig > 16) return false;
            w = w * 10 + (unsigned)(*p - '0');
        }
    }
    if (ndig == 0) return false;
    if (p < e && (*p == 'e' || *p == 'E')) {
        ++p;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) eneg = (*p++ == '-');
        const char *d0 = p;
        int x = 0;
        for (; p < e && *p >= '0' && *p <= '9'; ++p)
            if ((x = x * 10 + (*p - '0')) > 9999) return false;
        if (p == d0) return false;
        scale += eneg ? -x : x;
    }
    if (p != e || w > (1ull << 53)) return false;
    if (w == 0) {
        *v = neg ? -0.0 : 0.0;
        return true;
    }
    if (scale < -22 || scale > 22) return false;
    const double d = static_cast<double>(w);
    const double r = scale >= 0 ? d * kPow10[scale] : d / kPow10[-scale];
    *v = neg ? -r : r;
    return true;
}

bool parse_double(const char *tok, double *v)
{
    char *end = nullptr;
    const double r = std::strtod(tok, &end);   // fscanf "%lg" converts the same way
    if (end == tok || *end != '\0') return false;
    *v = r;
    return true;
}

void lower(char *s)
{
    for (; *s; ++s)
        if (*s >= 'A' && *s <= 'Z') *s = (char)(*s - 'A' + 'a');
}

// First line of f that is neither a comment nor blank, into line.
int next_content_line(FILE *f, char *line, size_t cap)
{
    for (;;) {
        if (std::fgets(line, (int)cap, f) == nullptr) return MM_PREMATURE_EOF;
        const char *p = line;
        while (*p && is_space(*p)) ++p;
        if (*p == '\0' || *p == '%') continue;
        return 0;
    }
}

// "M N [nz]" of the size line; nz may exceed the int range here.
int read_size_line(FILE *f, int nfields, long long out[3])
{
    char line[MM_MAX_LINE_LENGTH];
    const int rc = next_content_line(f, line, sizeof line);
    if (rc) return rc;
    const char *p = line;
    const char *e = line + std::strlen(line);
    char tok[MM_MAX_TOKEN_LENGTH];
    for (int i = 0; i < nfields; ++i) {
        const char *q = p;
        while (q < e && *q != '\n') ++q;
        if (!next_token(p, q, tok, sizeof tok) || !parse_ll(tok, &out[i]) || out[i] < 0)
            return MM_PREMATURE_EOF;
    }
    return 0;
}

struct Mapped {
    const char *base = nullptr;
    size_t size = 0;
    ~Mapped()
    {
        if (base) munmap(const_cast<char *>(base), size);
    }
};

struct ThreadResult {
    long long lines = 0;        // entry lines in the range
    long long offdiag = 0;      // stored off-diagonal entries (index < nnz)
    long long err_line = -1;    // index of the first bad entry (0-based), -1: none
    const char *err_what = nullptr;
};

}  // namespace
}  // namespace sblas

using namespace sblas;

extern "C" {

int mm_read_banner(FILE *f, MM_typecode *matcode)
{
    char line[MM_MAX_LINE_LENGTH];
    char tk[5][MM_MAX_TOKEN_LENGTH];
    (*matcode)[0] = (*matcode)[1] = (*matcode)[2] = ' ';
    (*matcode)[3] = 'G';
    if (f == nullptr || std::fgets(line, sizeof line, f) == nullptr) return MM_PREMATURE_EOF;
    const char *p = line;
    const char *e = line + std::strlen(line);
    for (int i = 0; i < 5; ++i)
        if (!next_token(p, e, tk[i], sizeof tk[i])) return MM_PREMATURE_EOF;
    for (int i = 1; i < 5; ++i) lower(tk[i]);
    if (std::strncmp(tk[0], MatrixMarketBanner, std::strlen(MatrixMarketBanner)) != 0)
        return MM_NO_HEADER;
    if (std::strcmp(tk[1], "matrix") != 0) return MM_UNSUPPORTED_TYPE;
    (*matcode)[0] = 'M';
    if (!std::strcmp(tk[2], "coordinate")) (*matcode)[1] = 'C';
    else if (!std::strcmp(tk[2], "array")) (*matcode)[1] = 'A';
    else return MM_UNSUPPORTED_TYPE;
    if (!std::strcmp(tk[3], "real")) (*matcode)[2] = 'R';
    else if (!std::strcmp(tk[3], "complex")) (*matcode)[2] = 'C';
    else if (!std::strcmp(tk[3], "pattern")) (*matcode)[2] = 'P';
    else if (!std::strcmp(tk[3], "integer")) (*matcode)[2] = 'I';
    else return MM_UNSUPPORTED_TYPE;
    if (!std::strcmp(tk[4], "general")) (*matcode)[3] = 'G';
    else if (!std::strcmp(tk[4], "symmetric")) (*matcode)[3] = 'S';
    else if (!std::strcmp(tk[4], "hermitian")) (*matcode)[3] = 'H';
    else if (!std::strcmp(tk[4], "skew-symmetric")) (*matcode)[3] = 'K';
    else return MM_UNSUPPORTED_TYPE;
    return 0;
}

int mm_read_mtx_crd_size(FILE *f, int *M, int *N, int *nz)
{
    if (M) *M = 0;
    if (N) *N = 0;
    if (nz) *nz = 0;
    if (f == nullptr || !M || !N || !nz) return MM_PREMATURE_EOF;
    long long v[3];
    const int rc = read_size_line(f, 3, v);
    if (rc) return rc;
    if (v[0] > INT_MAX || v[1] > INT_MAX || v[2] > INT_MAX) return MM_UNSUPPORTED_TYPE;
    *M = (int)v[0];
    *N = (int)v[1];
    *nz = (int)v[2];
    return 0;
}

int mm_read_mtx_array_size(FILE *f, int *M, int *N)
{
    if (M) *M = 0;
    if (N) *N = 0;
    if (f == nullptr || !M || !N) return MM_PREMATURE_EOF;
    long long v[3];
    const int rc = read_size_line(f, 2, v);
    if (rc) return rc;
    if (v[0] > INT_MAX || v[1] > INT_MAX) return MM_UNSUPPORTED_TYPE;
    *M = (int)v[0];
    *N = (int)v[1];
    return 0;
}

int mm_is_valid(MM_typecode matcode)
{
    if (!mm_is_matrix(matcode)) return 0;
    if (mm_is_dense(matcode) && mm_is_pattern(matcode)) return 0;
    if (mm_is_real(matcode) && mm_is_hermitian(matcode)) return 0;
    if (mm_is_pattern(matcode) && (mm_is_hermitian(matcode) || mm_is_skew(matcode))) return 0;
    return 1;
}

char *mm_typecode_to_str(MM_typecode matcode)
{
    const char *t1, *t2, *t3;
    if (!mm_is_matrix(matcode)) return nullptr;
    if (mm_is_sparse(matcode)) t1 = "coordinate";
    else if (mm_is_dense(matcode)) t1 = "array";
    else return nullptr;
    if (mm_is_real(matcode)) t2 = "real";
    else if (mm_is_complex(matcode)) t2 = "complex";
    else if (mm_is_pattern(matcode)) t2 = "pattern";
    else if (mm_is_integer(matcode)) t2 = "integer";
    else return nullptr;
    if (mm_is_general(matcode)) t3 = "general";
    else if (mm_is_symmetric(matcode)) t3 = "symmetric";
    else if (mm_is_hermitian(matcode)) t3 = "hermitian";
    else if (mm_is_skew(matcode)) t3 = "skew-symmetric";
    else return nullptr;
    const size_t len = 7 + std::strlen(t1) + 1 + std::strlen(t2) + 1 + std::strlen(t3) + 1;
    char *s = static_cast<char *>(std::malloc(len));
    if (s) std::snprintf(s, len, "matrix %s %s %s", t1, t2, t3);
    return s;
}

// Header of a coordinate file; *data_offset (when given) is the byte offset
// of the first line after the size line.
static int read_header(const char *path, sblas_mm_header *h, long long *data_offset)
{
    if (path == nullptr || h == nullptr) {
        set_error(SBLAS_ERR_ARG, "sblas_mm_read_header: null argument");
        return SBLAS_ERR_ARG;
    }
    std::memset(h, 0, sizeof *h);
    FILE *f = std::fopen(path, "rb");
    if (f == nullptr) {
        set_error(SBLAS_ERR_ARG, "cannot open %s: %s", path, std::strerror(errno));
        return SBLAS_ERR_ARG;
    }
    MM_typecode tc;
    int rc = mm_read_banner(f, &tc);
    if (rc) {
        std::fclose(f);
        set_error(SBLAS_ERR_FORMAT, "%s: no MatrixMarket banner (mmio code %d)", path, rc);
        return SBLAS_ERR_FORMAT;
    }
    std::memcpy(h->typecode, tc, 4);
    if (!mm_is_coordinate(tc) || mm_is_complex(tc) || !mm_is_valid(tc)) {
        std::fclose(f);
        char *ts = mm_typecode_to_str(tc);
        set_error(SBLAS_ERR_UNSUPPORTED, "%s: type '%s' not read (only real, integer or "
                  "pattern coordinate files are)", path, ts ? ts : "invalid");
        std::free(ts);
        return SBLAS_ERR_UNSUPPORTED;
    }
    long long v[3];
    rc = read_size_line(f, 3, v);
    if (rc == 0 && (v[0] > INT_MAX || v[1] > INT_MAX)) rc = MM_UNSUPPORTED_TYPE;
    if (rc) {
        std::fclose(f);
        set_error(SBLAS_ERR_FORMAT, "%s: bad size line (mmio code %d)", path, rc);
        return SBLAS_ERR_FORMAT;
    }
    h->m = (int)v[0];
    h->n = (int)v[1];
    h->nnz = v[2];
    if (data_offset) *data_offset = std::ftell(f);
    std::fclose(f);
    return SBLAS_OK;
}

int sblas_mm_read_header(const char *path, sblas_mm_header *h)
{
    clear_error();
    return read_header(path, h, nullptr);
}

int sblas_mm_read_coo(const char *path, int expand_symmetric, int nthreads, long long cap,
                      int *row, int *col, double *val, long long *count)
{
    clear_error();
    if (count) *count = 0;
    const bool write = row || col || val;
    if (count == nullptr || (write && !(row && col && val)) || cap < 0) {
        set_error(SBLAS_ERR_ARG, "sblas_mm_read_coo: count and either all or none of "
                  "row, col, val are required");
        return SBLAS_ERR_ARG;
    }
    sblas_mm_header h;
    long long off = 0;
    int rc = read_header(path, &h, &off);
    if (rc) return rc;
    const char field = h.typecode[2];
    const char sym = h.typecode[3];
    const bool mirror = expand_symmetric && sym != 'G';
    const double msign = (sym == 'K') ? -1.0 : 1.0;
    const long long nnz = h.nnz;

    Mapped map;
    const char *data = "";
    size_t len = 0;
    if (nnz > 0) {
        const int fd = ::open(path, O_RDONLY);
        struct stat st;
        if (fd < 0 || ::fstat(fd, &st) != 0) {
            if (fd >= 0) ::close(fd);
            set_error(SBLAS_ERR_ARG, "cannot open %s: %s", path, std::strerror(errno));
            return SBLAS_ERR_ARG;
        }
        map.size = (size_t)st.st_size;
        if (map.size > (size_t)off) {
            void *b = ::mmap(nullptr, map.size, PROT_READ, MAP_PRIVATE, fd, 0);
            if (b == MAP_FAILED) {
                ::close(fd);
                map.size = 0;
                set_error(SBLAS_ERR_ARG, "cannot map %s: %s", path, std::strerror(errno));
                return SBLAS_ERR_ARG;
            }
            map.base = static_cast<const char *>(b);
            ::madvise(b, map.size, MADV_SEQUENTIAL);
            data = map.base + off;
            len = map.size - (size_t)off;
        }
        ::close(fd);
    }

    // thread ranges at line starts
    int T = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
    T = std::max(1, std::min(T, 64));
    T = (int)std::max<size_t>(1, std::min<size_t>((size_t)T, len / (1u << 20) + 1));
    std::vector<size_t> lo(T + 1);
    lo[0] = 0;
    lo[T] = len;
    for (int t = 1; t < T; ++t) {
        size_t b = std::max(lo[t - 1], len * (size_t)t / (size_t)T);
        while (b < len && b > 0 && data[b - 1] != '\n') ++b;
        lo[t] = b;
    }
    std::vector<ThreadResult> res(T);
    auto for_lines = [&](int t, auto &&fn) {
        const char *p = data + lo[t];
        const char *end = data + lo[t + 1];
        while (p < end) {
            const char *e = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
            if (e == nullptr) e = end;
            const char *q = p;
            while (q < e && is_space(*q)) ++q;
            if (q < e && *q != '%')
                if (!fn(q, e)) return;
            p = e + 1;
        }
    };
    auto run = [&](auto &&body) {
        if (T == 1) {
            body(0);
            return;
        }
        std::vector<std::thread> th;
        th.reserve(T);
        for (int t = 0; t < T; ++t) th.emplace_back(body, t);
        for (auto &x : th) x.join();
    };

    // pass 1: entry lines per thread
    run([&](int t) {
        long long c = 0;
        for_lines(t, [&](const char *, const char *) {
            ++c;
            return true;
        });
        res[t].lines = c;
    });
    std::vector<long long> first(T + 1, 0);
    for (int t = 0; t < T; ++t) first[t + 1] = first[t] + res[t].lines;
    if (first[T] < nnz) {
        set_error(SBLAS_ERR_FORMAT, "%s: %lld entries announced, %lld found (premature end of "
                  "file)", path, nnz, first[T]);
        return SBLAS_ERR_FORMAT;
    }

    // pass 2: parse (entries below nnz), count off-diagonals
    const int m = h.m, n = h.n;
    run([&](int t) {
        long long k = first[t];
        long long od = 0;
        char tok[MM_MAX_TOKEN_LENGTH];
        for_lines(t, [&](const char *p, const char *e) {
            if (k >= nnz) return false;
            long long r, c;
            double v = 1.0;
            const char *bad = nullptr;
            if (!scan_ll(p, e, &r)) bad = "row index";
            else if (!scan_ll(p, e, &c)) bad = "column index";
            else if (r < 1 || r > m || c < 1 || c > n) bad = "index out of range";
            else if (field == 'R') {
                while (p < e && is_space(*p)) ++p;
                const char *t = p;
                while (t < e && !is_space(*t)) ++t;
                if (t > p && fast_double(p, t, &v)) {
                    p = t;
                } else if (t > p && t < data + len) {
                    // strtod in place: the byte after the token is whitespace
                    // inside the mapping, so the conversion stops there
                    char *end = nullptr;
                    v = std::strtod(p, &end);
                    if (end != t) bad = "value";
                    p = t;
                } else if (!next_token(p, e, tok, sizeof tok) || !parse_double(tok, &v)) {
                    bad = "value";
                }
            } else if (field == 'I') {
                long long iv;
                if (!scan_ll(p, e, &iv)) bad = "value";
                else v = (double)iv;
            }
            if (bad) {
                res[t].err_line = k;
                res[t].err_what = bad;
                return false;
            }
            if (write && k < cap) {
                row[k] = (int)(r - 1);
                col[k] = (int)(c - 1);
                val[k] = v;
            }
            od += (r != c);
            ++k;
            return true;
        });
        res[t].offdiag = od;
    });
    for (int t = 0; t < T; ++t)
        if (res[t].err_line >= 0) {
            set_error(SBLAS_ERR_FORMAT, "%s: entry %lld (data line after the size line): bad %s",
                      path, res[t].err_line + 1, res[t].err_what);
            return SBLAS_ERR_FORMAT;
        }
    std::vector<long long> mfirst(T + 1, 0);
    for (int t = 0; t < T; ++t) mfirst[t + 1] = mfirst[t] + (mirror ? res[t].offdiag : 0);
    const long long total = nnz + mfirst[T];
    *count = total;
    if (!write) return SBLAS_OK;
    if (cap < total) {
        set_error(SBLAS_ERR_ARG, "sblas_mm_read_coo: cap %lld < %lld entries", cap, total);
        return SBLAS_ERR_ARG;
    }

    // pass 3: mirrors of each thread's stored entries, after all stored ones
    if (mirror) {
        run([&](int t) {
            const long long b = std::min(first[t], nnz), e = std::min(first[t + 1], nnz);
            long long o = nnz + mfirst[t];
            for (long long k = b; k < e; ++k)
                if (row[k] != col[k]) {
                    row[o] = col[k];
                    col[o] = row[k];
                    val[o] = msign * val[k];
                    ++o;
                }
        });
    }
    return SBLAS_OK;
}

}  // extern "C"
