/*
 * gpr_tops.cpp -- tops.txt without the external sort.  The reference's run
 * script keeps the best samples with
 *     sort -g -k3 --parallel=8 samples.txt | tail -n 10000 > tops.txt
 * (run-all.sh:45).  This keeps, while the lines are produced, exactly the
 * lines that command prints (in the C locale), in its order:
 *
 *  - the key of a line starts at its third field, fields being separated by
 *    the empty string before a run of blanks (no -t, no -b: the blanks belong
 *    to the field that follows them);
 *  - -g reads the key with strtold: keys that are not numbers sort first
 *    (among themselves equal), then NaNs, then numbers in numeric order with
 *    -0 == +0;
 *  - lines with equal keys are ordered by their bytes (the last-resort
 *    comparison), shorter first on a common prefix;
 *  - `tail -n K` keeps the K largest lines under that order.
 *
 * Note that the header lines of samples.txt take part: "# \tSeed: S",
 * "# \tBlocks: B", "# \tGPU: G" and every data line "# \tx\ty\tsd" have a
 * numeric third field, so they rank among the samples exactly as the run
 * script ranks them.  NaN keys are taken as equal to one another (sort
 * orders NaNs by their bit pattern, which depends on the long double format).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/gpuropolis_host.h"

namespace {

struct Entry {
    int cls;            /* 0: no number, 1: NaN, 2: number */
    long double key;
    std::string line;
};

bool is_blank(unsigned char c) { return c == ' ' || c == '\t' || c == '\n'; }

Entry make_entry(const char* s, size_t n) {
    Entry e;
    e.line.assign(s, n);
    const char* p = e.line.c_str();
    const char* lim = p + n;
    for (int f = 0; f < 2 && p < lim; ++f) {      /* skip fields 1 and 2 */
        while (p < lim && is_blank((unsigned char)*p)) ++p;
        while (p < lim && !is_blank((unsigned char)*p)) ++p;
    }
    char* end = nullptr;
    const long double v = strtold(p, &end);
    if (end == p) { e.cls = 0; e.key = 0.0L; }
    else if (v != v) { e.cls = 1; e.key = 0.0L; }
    else { e.cls = 2; e.key = v; }
    return e;
}

/* a < b in the order of sort -g -k3 */
bool entry_less(const Entry& a, const Entry& b) {
    if (a.cls != b.cls) return a.cls < b.cls;
    if (a.cls == 2) {
        if (a.key < b.key) return true;
        if (b.key < a.key) return false;
    }
    return a.line < b.line;
}

}  // namespace

struct gpr_tops {
    int k;
    std::vector<Entry> pool;
    void prune() {
        if ((int)pool.size() <= k) return;
        std::nth_element(pool.begin(), pool.begin() + (pool.size() - k), pool.end(), entry_less);
        pool.erase(pool.begin(), pool.begin() + (pool.size() - k));
    }
    void offer(const char* s, size_t n) {
        pool.push_back(make_entry(s, n));
        if ((int)pool.size() >= 2 * k + 1024) prune();
    }
};

extern "C" {

gpr_tops* gpr_tops_new(int k) {
    if (k < 1) return nullptr;
    gpr_tops* t = new gpr_tops();
    t->k = k;
    return t;
}

void gpr_tops_free(gpr_tops* t) { delete t; }

int gpr_tops_add_text(gpr_tops* t, const char* text, int64_t len) {
    if (!t || len < 0 || (len > 0 && !text)) return GPR_HOST_ERR_ARG;
    int64_t a = 0;
    while (a < len) {
        const char* nl = (const char*)memchr(text + a, '\n', (size_t)(len - a));
        const int64_t b = nl ? (int64_t)(nl - text) : len;
        t->offer(text + a, (size_t)(b - a));
        a = b + 1;
    }
    return GPR_HOST_OK;
}

int gpr_tops_add_lines(gpr_tops* t, const char* text, int64_t len, const int* lines, int n) {
    if (!t || len < 0 || n < 0 || (n > 0 && (!text || !lines))) return GPR_HOST_ERR_ARG;
    int64_t a = 0;
    int line = 0;
    for (int i = 0; i < n; ++i) {
        if (lines[i] < line) return GPR_HOST_ERR_ARG;   /* ascending, no repeats */
        while (line < lines[i] && a < len) {
            const char* nl = (const char*)memchr(text + a, '\n', (size_t)(len - a));
            if (!nl) return GPR_HOST_ERR_ARG;
            a = (int64_t)(nl - text) + 1;
            ++line;
        }
        if (a >= len) return GPR_HOST_ERR_ARG;
        const char* nl = (const char*)memchr(text + a, '\n', (size_t)(len - a));
        const int64_t b = nl ? (int64_t)(nl - text) : len;
        t->offer(text + a, (size_t)(b - a));
        a = b + 1;
        ++line;
    }
    return GPR_HOST_OK;
}

int64_t gpr_tops_write(gpr_tops* t, const char* path) {
    if (!t || !path) return -1;
    t->prune();
    std::sort(t->pool.begin(), t->pool.end(), entry_less);
    FILE* fp = fopen(path, "w");
    if (!fp) return -1;
    for (const Entry& e : t->pool) {
        fwrite(e.line.data(), 1, e.line.size(), fp);
        fputc('\n', fp);
    }
    const bool ok = fclose(fp) == 0;
    return ok ? (int64_t)t->pool.size() : -1;
}

}  /* extern "C" */
