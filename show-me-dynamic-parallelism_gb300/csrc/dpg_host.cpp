// Host-side graph I/O and construction for the dpg library.
//
// Follows common/global.cpp of the reference:
//   readInputDIMACS9   global.cpp:29-64    -> read_dimacs9
//   readInputDIMACS10  global.cpp:66-105   -> read_dimacs10
//   readInputSLNDC     global.cpp:107-190  -> read_slndc
//   convertCSR         global.cpp:192-235  -> dpg_csr_from_arcs (per-vertex order reversed)
//   invertGraph        global.cpp:237-277  -> dpg_csr_transpose
//   outputCost/Level/Rank/Color global.cpp:361-399 -> dpg_write_*
// The reference keeps one std::list per vertex and pops from the back; here a counting sort that
// fills each vertex's slice from its end gives the same arrays in O(V+E) with flat memory.
// Unlike the reference, malformed input is reported as DPG_ERR_FORMAT instead of exit()/UB.

#include "dpg_internal.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#include <algorithm>
#include <cerrno>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace dpg {

namespace {

// glibc's random()/rand() additive-feedback generator (TYPE_3: degree 31, separation 3), seeded
// the way srandom() seeds it. The reference draws DIMACS10/SLNDC weights with srand(7) and
// rand() % 1000 + 1 (global.cpp:84,98,167,180); this reproduces that stream without touching the
// process-wide rand() state.
class GlibcRandom {
public:
    explicit GlibcRandom(uint32_t seed) {
        int32_t r[34];
        r[0] = static_cast<int32_t>(seed == 0 ? 1 : seed);
        for (int i = 1; i < 31; ++i) {
            // r[i] = (16807 * r[i-1]) % 2147483647 computed without overflow (Schrage).
            const int32_t hi = r[i - 1] / 127773;
            const int32_t lo = r[i - 1] % 127773;
            int32_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            r[i] = word;
        }
        for (int i = 0; i < 31; ++i) state_[i] = static_cast<uint32_t>(r[i]);
        f_ = 3;
        b_ = 0;
        for (int i = 0; i < 310; ++i) next();
    }
    int32_t next() {
        state_[f_] += state_[b_];
        const int32_t result = static_cast<int32_t>(state_[f_] >> 1);
        f_ = (f_ + 1) % 31;
        b_ = (b_ + 1) % 31;
        return result;
    }

private:
    uint32_t state_[31];
    int f_, b_;
};

// Line reader with the reference's buffer semantics (fgets into a BUFF_SIZE buffer).
constexpr size_t kLineBuf = 1024000;  // BUFF_SIZE, common/global.h:15

struct FileCloser {
    FILE* f;
    ~FileCloser() {
        if (f) fclose(f);
    }
};

bool parse_int_token(const char* p, long long* out) {
    // atoi-like: leading whitespace, optional sign, digits; trailing junk ignored like atoi.
    while (*p == ' ' || *p == '\t') ++p;
    char* end = nullptr;
    errno = 0;
    long long v = strtoll(p, &end, 10);
    if (end == p || errno != 0) return false;
    *out = v;
    return true;
}

// Tokenise on ' ' like strtok(buff, " ") (the reference's separator set is a single space).
void split_spaces(char* s, std::vector<char*>* toks) {
    toks->clear();
    char* save = nullptr;
    for (char* t = strtok_r(s, " ", &save); t != nullptr; t = strtok_r(nullptr, " ", &save))
        toks->push_back(t);
}

struct ArcList {
    int32_t V = 0;
    int64_t E = 0;
    int32_t source = 0;
    std::vector<int32_t> src, dst, w;  // arcs in adjacency-list push order
};

dpg_status read_dimacs9(FILE* fp, ArcList* g) {
    std::vector<char> buf(kLineBuf);
    std::vector<char*> toks;
    bool have_p = false;
    int64_t declared_e = 0;
    while (fgets(buf.data(), static_cast<int>(kLineBuf), fp) != nullptr) {
        char* line = buf.data();
        if (line[0] == 'c') continue;
        if (line[0] == 'p') {
            // strtok(buff+4, " "): skips "p sp" and reads node and arc counts.
            if (strlen(line) < 4) return set_error(DPG_ERR_FORMAT, "short 'p' line");
            split_spaces(line + 4, &toks);
            long long n = 0, m = 0;
            if (toks.size() < 2 || !parse_int_token(toks[0], &n) || !parse_int_token(toks[1], &m) ||
                n < 0 || m < 0 || n > INT32_MAX || m > INT64_MAX / 2)
                return set_error(DPG_ERR_FORMAT, "bad 'p' line");
            g->V = static_cast<int32_t>(n);
            declared_e = m;
            have_p = true;
            g->src.reserve(static_cast<size_t>(m));
            g->dst.reserve(static_cast<size_t>(m));
            g->w.reserve(static_cast<size_t>(m));
        }
        if (line[0] == 's') {
            split_spaces(line + 1, &toks);
            long long s = 0;
            if (toks.empty() || !parse_int_token(toks[0], &s)) return set_error(DPG_ERR_FORMAT, "bad 's' line");
            g->source = static_cast<int32_t>(s - 1);
        }
        if (line[0] == 'a') {
            if (!have_p) return set_error(DPG_ERR_FORMAT, "'a' line before 'p' line");
            split_spaces(line + 1, &toks);
            long long t = 0, h = 0, wt = 0;
            if (toks.size() < 3 || !parse_int_token(toks[0], &t) || !parse_int_token(toks[1], &h) ||
                !parse_int_token(toks[2], &wt))
                return set_error(DPG_ERR_FORMAT, "bad 'a' line");
            if (t < 1 || t > g->V || h < 1 || h > g->V)
                return set_error(DPG_ERR_FORMAT, "arc endpoint out of range");
            if (wt < INT32_MIN || wt > INT32_MAX) return set_error(DPG_ERR_FORMAT, "weight out of int32 range");
            g->src.push_back(static_cast<int32_t>(t - 1));
            g->dst.push_back(static_cast<int32_t>(h - 1));
            g->w.push_back(static_cast<int32_t>(wt));
        }
    }
    if (!have_p) return set_error(DPG_ERR_FORMAT, "missing 'p' line");
    g->E = static_cast<int64_t>(g->src.size());
    if (g->E != declared_e) return set_error(DPG_ERR_FORMAT, "arc count differs from the 'p' line");
    if (g->V > 0 && (g->source < 0 || g->source >= g->V))
        return set_error(DPG_ERR_FORMAT, "source vertex out of range");
    return DPG_OK;
}

// The same DIMACS9 reader over the whole file held in memory, in parallel. The file is cut into
// chunks at line boundaries; every thread runs the serial reader's per-line code (the same token
// splitting and atoi-like parsing) over its lines; the arcs are joined in file order. Shapes whose
// semantics depend on line order beyond that (several 'p' lines, a line longer than the serial
// reader's buffer) return false so that the caller runs the serial reader instead.
struct ChunkArcs {
    std::vector<int32_t> src, dst, w;  // 1-based endpoints as read, range-checked after the join
    std::vector<int64_t> arc_pos;      // byte position of each arc line (for the first range error)
    int64_t err_pos = INT64_MAX;
    std::string err;
    std::vector<std::pair<int64_t, std::pair<long long, long long>>> p_lines;  // (pos, (V, E))
    int64_t s_pos = -1;
    long long s_val = 0;
    int64_t first_a = INT64_MAX;
};

bool read_dimacs9_parallel(char* buf, int64_t n, int threads, ArcList* g, dpg_status* status) {
    // Longest line check (the serial reader's fgets splits lines of kLineBuf - 1 characters or more).
    std::vector<int64_t> cut(static_cast<size_t>(threads) + 1, n);
    cut[0] = 0;
    for (int t = 1; t < threads; ++t) {
        int64_t c = n * t / threads;
        while (c < n && buf[c - 1] != '\n') ++c;
        cut[t] = std::max(c, cut[t - 1]);
    }
    std::vector<ChunkArcs> part(static_cast<size_t>(threads));
    bool too_long = false;
#pragma omp parallel for num_threads(threads) schedule(static, 1) reduction(|| : too_long)
    for (int t = 0; t < threads; ++t) {
        ChunkArcs& R = part[t];
        std::vector<char*> toks;
        const size_t guess = static_cast<size_t>((cut[t + 1] - cut[t]) / 12 + 16);
        R.src.reserve(guess);
        R.dst.reserve(guess);
        R.w.reserve(guess);
        R.arc_pos.reserve(guess);
        int64_t pos = cut[t];
        while (pos < cut[t + 1]) {
            int64_t end = pos;
            while (end < cut[t + 1] && buf[end] != '\n') ++end;
            if (end - pos + 1 >= static_cast<int64_t>(kLineBuf) - 1) too_long = true;
            const int64_t next = end + 1;
            char saved = end < n ? buf[end] : 0;
            if (end < n) buf[end] = 0;
            char* line = buf + pos;
            if (R.err_pos == INT64_MAX && !too_long) {
                if (line[0] == 'p') {
                    long long V = 0, E = 0;
                    if (strlen(line) < 4) {
                        R.err_pos = pos;
                        R.err = "short 'p' line";
                    } else {
                        split_spaces(line + 4, &toks);
                        if (toks.size() < 2 || !parse_int_token(toks[0], &V) || !parse_int_token(toks[1], &E) ||
                            V < 0 || E < 0 || V > INT32_MAX || E > INT64_MAX / 2) {
                            R.err_pos = pos;
                            R.err = "bad 'p' line";
                        } else {
                            R.p_lines.push_back({pos, {V, E}});
                        }
                    }
                } else if (line[0] == 's') {
                    split_spaces(line + 1, &toks);
                    long long sv = 0;
                    if (toks.empty() || !parse_int_token(toks[0], &sv)) {
                        R.err_pos = pos;
                        R.err = "bad 's' line";
                    } else {
                        R.s_pos = pos;
                        R.s_val = sv;
                    }
                } else if (line[0] == 'a') {
                    if (R.first_a == INT64_MAX) R.first_a = pos;
                    split_spaces(line + 1, &toks);
                    long long a = 0, h = 0, wt = 0;
                    if (toks.size() < 3 || !parse_int_token(toks[0], &a) || !parse_int_token(toks[1], &h) ||
                        !parse_int_token(toks[2], &wt)) {
                        R.err_pos = pos;
                        R.err = "bad 'a' line";
                    } else if (a < 1 || a > INT32_MAX || h < 1 || h > INT32_MAX) {
                        R.err_pos = pos;
                        R.err = "arc endpoint out of range";
                    } else if (wt < INT32_MIN || wt > INT32_MAX) {
                        R.err_pos = pos;
                        R.err = "weight out of int32 range";
                    } else {
                        R.src.push_back(static_cast<int32_t>(a));
                        R.dst.push_back(static_cast<int32_t>(h));
                        R.w.push_back(static_cast<int32_t>(wt));
                        R.arc_pos.push_back(pos);
                    }
                }
            }
            if (end < n) buf[end] = saved;
            pos = next;
        }
    }
    if (too_long) return false;
    int np = 0;
    int64_t p_pos = INT64_MAX, first_a = INT64_MAX, err_pos = INT64_MAX, s_pos = -1;
    long long V = 0, declared = 0, s_val = 1;
    std::string err;
    for (const ChunkArcs& R : part) {
        np += static_cast<int>(R.p_lines.size());
        for (auto& pl : R.p_lines) {
            p_pos = pl.first;
            V = pl.second.first;
            declared = pl.second.second;
        }
        first_a = std::min(first_a, R.first_a);
        if (R.err_pos < err_pos) {
            err_pos = R.err_pos;
            err = R.err;
        }
        if (R.s_pos > s_pos) {
            s_pos = R.s_pos;
            s_val = R.s_val;
        }
    }
    if (np > 1) return false;
    // The serial reader stops at the first failing line in file order.
    if (np == 1 && first_a < p_pos && first_a < err_pos) {
        err_pos = first_a;
        err = "'a' line before 'p' line";
    }
    if (np == 0 && first_a < err_pos) {
        err_pos = first_a;
        err = "'a' line before 'p' line";
    }
    // Endpoint range against V: the first out-of-range arc line in file order.
    for (const ChunkArcs& R : part) {
        bool found = false;
        for (size_t k = 0; k < R.src.size() && R.arc_pos[k] < err_pos; ++k) {
            if (R.src[k] > V || R.dst[k] > V) {
                err_pos = R.arc_pos[k];
                err = "arc endpoint out of range";
                found = true;
                break;
            }
        }
        if (found) break;
    }
    if (err_pos != INT64_MAX) {
        *status = set_error(DPG_ERR_FORMAT, err);
        return true;
    }
    if (np == 0) {
        *status = set_error(DPG_ERR_FORMAT, "missing 'p' line");
        return true;
    }
    int64_t total = 0;
    std::vector<int64_t> at(part.size() + 1, 0);
    for (size_t t = 0; t < part.size(); ++t) at[t + 1] = at[t] + static_cast<int64_t>(part[t].src.size());
    total = at.back();
    g->V = static_cast<int32_t>(V);
    g->source = static_cast<int32_t>(s_val - 1);
    g->src.resize(static_cast<size_t>(total));
    g->dst.resize(static_cast<size_t>(total));
    g->w.resize(static_cast<size_t>(total));
#pragma omp parallel for num_threads(threads) schedule(static, 1)
    for (int t = 0; t < static_cast<int>(part.size()); ++t) {
        const ChunkArcs& R = part[t];
        for (size_t k = 0; k < R.src.size(); ++k) {
            g->src[at[t] + k] = R.src[k] - 1;
            g->dst[at[t] + k] = R.dst[k] - 1;
            g->w[at[t] + k] = R.w[k];
        }
    }
    g->E = total;
    if (g->E != declared) {
        *status = set_error(DPG_ERR_FORMAT, "arc count differs from the 'p' line");
        return true;
    }
    if (g->V > 0 && (g->source < 0 || g->source >= g->V)) {
        *status = set_error(DPG_ERR_FORMAT, "source vertex out of range");
        return true;
    }
    *status = DPG_OK;
    return true;
}

dpg_status read_dimacs10(FILE* fp, ArcList* g) {
    std::vector<char> buf(kLineBuf);
    std::vector<char*> toks;
    bool got = false;
    while (fgets(buf.data(), static_cast<int>(kLineBuf), fp) != nullptr) {
        if (buf[0] == '%') continue;
        got = true;
        break;
    }
    if (!got) return set_error(DPG_ERR_FORMAT, "missing DIMACS10 header");
    split_spaces(buf.data(), &toks);
    long long n = 0, m = 0;
    if (toks.size() < 2 || !parse_int_token(toks[0], &n) || !parse_int_token(toks[1], &m) || n < 0 ||
        m < 0 || n > INT32_MAX)
        return set_error(DPG_ERR_FORMAT, "bad DIMACS10 header");
    g->V = static_cast<int32_t>(n);
    const int64_t declared_e = 2 * m;  // noEdgeTotal = 2 * noEdgeTotal (global.cpp:80)
    GlibcRandom rng(7);                // srand(7), global.cpp:84
    for (int32_t i = 0; i < g->V; ++i) {
        if (fgets(buf.data(), static_cast<int>(kLineBuf), fp) == nullptr)
            return set_error(DPG_ERR_FORMAT, "Parsing adjacencylist fails!");
        if (strlen(buf.data()) == kLineBuf - 1) return set_error(DPG_ERR_FORMAT, "adjacency line too long");
        split_spaces(buf.data(), &toks);
        for (char* p : toks) {
            if (*p == '\n') break;  // while (p!=NULL && (*p)!='\n')
            long long h = 0;
            if (!parse_int_token(p, &h)) return set_error(DPG_ERR_FORMAT, "bad neighbour id");
            if (h < 1 || h > g->V) return set_error(DPG_ERR_FORMAT, "neighbour id out of range");
            g->src.push_back(i);
            g->dst.push_back(static_cast<int32_t>(h - 1));
            g->w.push_back(rng.next() % 1000 + 1);
        }
    }
    g->E = static_cast<int64_t>(g->src.size());
    if (g->E != declared_e) return set_error(DPG_ERR_FORMAT, "neighbour count differs from 2*header edges");
    g->source = 0;
    return DPG_OK;
}

dpg_status read_slndc(FILE* fp, ArcList* g) {
    char line[256];
    if (fgets(line, 256, fp) == nullptr) return set_error(DPG_ERR_FORMAT, "missing SLNDC header");
    if (fgets(line, 256, fp) == nullptr) return set_error(DPG_ERR_FORMAT, "missing SLNDC header");
    if (fgets(line, 256, fp) == nullptr) return set_error(DPG_ERR_FORMAT, "Parsing total node number fails!");
    if (strlen(line) < 9) return set_error(DPG_ERR_FORMAT, "bad SLNDC node line");
    std::vector<char*> toks;
    split_spaces(line + 9, &toks);  // strtok(buff+9, " ")
    long long n = 0;
    if (toks.empty() || !parse_int_token(toks[0], &n) || n < 0 || n > INT32_MAX / 2)
        return set_error(DPG_ERR_FORMAT, "bad SLNDC node count");
    if (fgets(line, 256, fp) == nullptr) return set_error(DPG_ERR_FORMAT, "missing SLNDC header");
    const int64_t cap = 2 * n;  // tempNodeList / mapTable sized noNodeTotal*2 (global.cpp:133-134)
    std::vector<std::vector<int32_t>> temp(static_cast<size_t>(cap));
    std::vector<int32_t> map(static_cast<size_t>(cap), 0);
    int64_t max_id = -1;
    int64_t count = 0;
    for (;;) {
        int t = 0, h = 0;
        int r = fscanf(fp, "%d%d", &t, &h);
        if (r == EOF) break;
        if (r != 2) return set_error(DPG_ERR_FORMAT, "bad SLNDC edge line");
        if (t < 0 || h < 0 || t >= cap || h >= cap) return set_error(DPG_ERR_FORMAT, "SLNDC node id out of range");
        map[t] = map[h] = 1;
        if (t > max_id) max_id = t;
        if (h > max_id) max_id = h;
        temp[t].push_back(h);
        ++count;
    }
    int32_t nv = 0;
    for (int64_t i = 0; i <= max_id; ++i) map[i] = map[i] == 1 ? nv++ : -1;
    g->V = nv;
    GlibcRandom rng(7);  // srand(7), global.cpp:167
    g->src.reserve(static_cast<size_t>(count));
    g->dst.reserve(static_cast<size_t>(count));
    g->w.reserve(static_cast<size_t>(count));
    for (int64_t i = 0; i <= max_id; ++i) {
        if (map[i] == -1) continue;
        for (int32_t head : temp[i]) {  // pop_front order == file order
            g->src.push_back(map[i]);
            g->dst.push_back(map[head]);
            g->w.push_back(rng.next() % 1000 + 1);
        }
    }
    g->E = count;
    g->source = 0;
    return DPG_OK;
}

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t counter) {
    return splitmix64(splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + counter);
}

// Seeded bijection of [0, 2^bits): odd multiplications and xor-shifts are each invertible modulo
// 2^bits, so their composition is a permutation.
inline uint32_t permute_id(uint32_t x, int bits, uint64_t seed) {
    if (bits <= 0) return x;
    const uint64_t mask = (bits >= 32) ? 0xFFFFFFFFull : ((1ull << bits) - 1);
    uint64_t y = x;
    const int sh = bits / 2 + 1;
    for (int round = 0; round < 3; ++round) {
        const uint64_t k = draw(seed, 0xA5A5ull + round, 0);
        y = (y ^ (k >> 40)) & mask;
        y = (y * ((k & 0xFFFFFFFFull) | 1ull)) & mask;
        if (sh < bits) y = (y ^ (y >> sh)) & mask;
    }
    return static_cast<uint32_t>(y);
}

}  // namespace

}  // namespace dpg

using namespace dpg;

extern "C" {

dpg_status dpg_csr_from_arcs(int32_t V, int64_t E, const int32_t* src, const int32_t* dst,
                             const int32_t* w, int32_t* offsets, int32_t* col, int32_t* weights) {
    if (V < 0 || E < 0 || E > INT32_MAX || !offsets || (E > 0 && (!src || !dst || !col)))
        return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_from_arcs: bad sizes or null pointers");
    if (weights && !w && E > 0) return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_from_arcs: weights out without weights in");
    std::vector<int64_t> cnt(static_cast<size_t>(V) + 1, 0);
    for (int64_t e = 0; e < E; ++e) {
        if (src[e] < 0 || src[e] >= V || dst[e] < 0 || dst[e] >= V)
            return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_from_arcs: arc endpoint out of range");
        ++cnt[src[e]];
    }
    int64_t acc = 0;
    for (int32_t v = 0; v < V; ++v) {
        offsets[v] = static_cast<int32_t>(acc);
        acc += cnt[v];
        cnt[v] = acc;  // cursor starts at the end of v's slice
    }
    offsets[V] = static_cast<int32_t>(acc);
    // convertCSR pops each adjacency list from the back: the last arc read is first in the row.
    for (int64_t e = 0; e < E; ++e) {
        const int64_t pos = --cnt[src[e]];
        col[pos] = dst[e];
        if (weights) weights[pos] = w[e];
    }
    return DPG_OK;
}

dpg_status dpg_csr_transpose_perm(int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                                  int32_t* in_offsets, int32_t* in_col, int32_t* in_arc) {
    if (V < 0 || E < 0 || E > INT32_MAX || !offsets || !in_offsets || (E > 0 && (!col || !in_col)))
        return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_transpose: bad sizes or null pointers");
    if (offsets[0] != 0 || offsets[V] != E) return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_transpose: offsets do not span E");
    std::vector<int64_t> cnt(static_cast<size_t>(V) + 1, 0);
    for (int64_t e = 0; e < E; ++e) {
        if (col[e] < 0 || col[e] >= V) return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_transpose: column out of range");
        ++cnt[col[e]];
    }
    int64_t acc = 0;
    for (int32_t v = 0; v < V; ++v) {
        in_offsets[v] = static_cast<int32_t>(acc);
        acc += cnt[v];
        cnt[v] = acc;
    }
    in_offsets[V] = static_cast<int32_t>(acc);
    // invertGraph pushes i onto child list of col[j] for i ascending, j ascending, then pops from
    // the back: the row of v lists its in-neighbours in the reverse of that push order.
    for (int32_t i = 0; i < V; ++i) {
        if (offsets[i + 1] < offsets[i]) return set_error(DPG_ERR_INVALID_ARG, "dpg_csr_transpose: offsets decrease");
        for (int32_t j = offsets[i]; j < offsets[i + 1]; ++j) {
            const int64_t pos = --cnt[col[j]];
            in_col[pos] = i;
            if (in_arc) in_arc[pos] = j;
        }
    }
    return DPG_OK;
}

dpg_status dpg_csr_transpose(int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                             int32_t* in_offsets, int32_t* in_col) {
    return dpg_csr_transpose_perm(V, E, offsets, col, in_offsets, in_col, nullptr);
}

dpg_status dpg_read_graph(const char* path, int32_t format, dpg_host_graph* out) {
    return dpg_read_graph_ex(path, format, 0, out);
}

dpg_status dpg_read_graph_ex(const char* path, int32_t format, int32_t threads, dpg_host_graph* out) {
    if (!path || !out) return set_error(DPG_ERR_INVALID_ARG, "dpg_read_graph: null argument");
    if (threads < 0) return set_error(DPG_ERR_INVALID_ARG, "threads must be >= 0");
    memset(out, 0, sizeof(*out));
    FILE* fp = fopen(path, "r");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot open ") + path);
    FileCloser closer{fp};
    ArcList arcs;
    dpg_status st = DPG_OK;
    bool done = false;
#ifdef _OPENMP
    const int nth = threads > 0 ? threads : omp_get_max_threads();
#else
    const int nth = 1;
#endif
    if (format == 0 && nth > 1 && fseek(fp, 0, SEEK_END) == 0) {
        // Whole file in memory, then the parallel reader (identical results).
        const long long n = ftell(fp);
        if (n > 0 && fseek(fp, 0, SEEK_SET) == 0) {
            std::vector<char> buf(static_cast<size_t>(n) + 1, 0);
            if (fread(buf.data(), 1, static_cast<size_t>(n), fp) == static_cast<size_t>(n))
                done = read_dimacs9_parallel(buf.data(), n, nth, &arcs, &st);
        }
        if (!done) {
            arcs = ArcList();
            rewind(fp);
        }
    }
    if (!done) {
        switch (format) {
            case 0: st = read_dimacs9(fp, &arcs); break;
            case 1: st = read_dimacs10(fp, &arcs); break;
            case 2: st = read_slndc(fp, &arcs); break;
            default: return set_error(DPG_ERR_INVALID_ARG, "Wrong code for dataset");
        }
    }
    if (st != DPG_OK) return st;
    if (arcs.E > INT32_MAX) return set_error(DPG_ERR_CAPACITY, "more than 2^31-1 arcs");
    out->V = arcs.V;
    out->E = arcs.E;
    out->source = arcs.source;
    out->offsets = static_cast<int32_t*>(malloc(sizeof(int32_t) * (static_cast<size_t>(arcs.V) + 1)));
    out->col = static_cast<int32_t*>(malloc(sizeof(int32_t) * static_cast<size_t>(arcs.E > 0 ? arcs.E : 1)));
    out->weights = static_cast<int32_t*>(malloc(sizeof(int32_t) * static_cast<size_t>(arcs.E > 0 ? arcs.E : 1)));
    if (!out->offsets || !out->col || !out->weights) {
        dpg_host_graph_free(out);
        return set_error(DPG_ERR_CAPACITY, "host allocation failed");
    }
    st = dpg_csr_from_arcs(arcs.V, arcs.E, arcs.src.data(), arcs.dst.data(), arcs.w.data(), out->offsets,
                           out->col, out->weights);
    if (st != DPG_OK) dpg_host_graph_free(out);
    return st;
}

// Binary CSR cache: "DPGCSR01", int32 V, int64 E, int32 source, int32 has_weights, then offsets
// [V+1], col [E] and (if present) weights [E], all little-endian int32.
static const char kCacheMagic[8] = {'D', 'P', 'G', 'C', 'S', 'R', '0', '1'};

dpg_status dpg_write_graph_cache(const char* path, const dpg_host_graph* g) {
    if (!path || !g || !g->offsets || (g->E > 0 && !g->col)) return set_error(DPG_ERR_INVALID_ARG, "null argument");
    FILE* fp = fopen(path, "wb");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot open ") + path);
    FileCloser closer{fp};
    const int32_t hw = g->weights ? 1 : 0;
    bool ok = fwrite(kCacheMagic, 1, 8, fp) == 8 && fwrite(&g->V, 4, 1, fp) == 1 && fwrite(&g->E, 8, 1, fp) == 1 &&
              fwrite(&g->source, 4, 1, fp) == 1 && fwrite(&hw, 4, 1, fp) == 1 &&
              fwrite(g->offsets, 4, static_cast<size_t>(g->V) + 1, fp) == static_cast<size_t>(g->V) + 1 &&
              fwrite(g->col, 4, static_cast<size_t>(g->E), fp) == static_cast<size_t>(g->E) &&
              (!hw || fwrite(g->weights, 4, static_cast<size_t>(g->E), fp) == static_cast<size_t>(g->E));
    if (!ok) return set_error(DPG_ERR_IO, std::string("write failed: ") + path);
    return DPG_OK;
}

dpg_status dpg_read_graph_cache(const char* path, dpg_host_graph* out) {
    if (!path || !out) return set_error(DPG_ERR_INVALID_ARG, "null argument");
    memset(out, 0, sizeof(*out));
    FILE* fp = fopen(path, "rb");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot open ") + path);
    FileCloser closer{fp};
    char magic[8];
    int32_t V = 0, source = 0, hw = 0;
    int64_t E = 0;
    if (fread(magic, 1, 8, fp) != 8 || memcmp(magic, kCacheMagic, 8) != 0 || fread(&V, 4, 1, fp) != 1 ||
        fread(&E, 8, 1, fp) != 1 || fread(&source, 4, 1, fp) != 1 || fread(&hw, 4, 1, fp) != 1 || V < 0 || E < 0 ||
        E > INT32_MAX || (hw != 0 && hw != 1))
        return set_error(DPG_ERR_FORMAT, std::string("not a graph cache: ") + path);
    out->V = V;
    out->E = E;
    out->source = source;
    out->offsets = static_cast<int32_t*>(malloc(4 * (static_cast<size_t>(V) + 1)));
    out->col = static_cast<int32_t*>(malloc(4 * static_cast<size_t>(E > 0 ? E : 1)));
    out->weights = static_cast<int32_t*>(malloc(4 * static_cast<size_t>(E > 0 ? E : 1)));
    if (!out->offsets || !out->col || !out->weights) {
        dpg_host_graph_free(out);
        return set_error(DPG_ERR_CAPACITY, "host allocation failed");
    }
    bool ok = fread(out->offsets, 4, static_cast<size_t>(V) + 1, fp) == static_cast<size_t>(V) + 1 &&
              fread(out->col, 4, static_cast<size_t>(E), fp) == static_cast<size_t>(E);
    if (ok && hw) ok = fread(out->weights, 4, static_cast<size_t>(E), fp) == static_cast<size_t>(E);
    else if (ok) memset(out->weights, 0, 4 * static_cast<size_t>(E > 0 ? E : 1));
    if (ok && (out->offsets[0] != 0 || out->offsets[V] != E)) ok = false;
    if (!ok) {
        dpg_host_graph_free(out);
        return set_error(DPG_ERR_FORMAT, std::string("truncated or inconsistent graph cache: ") + path);
    }
    return DPG_OK;
}

void dpg_host_graph_free(dpg_host_graph* g) {
    if (!g) return;
    free(g->offsets);
    free(g->col);
    free(g->weights);
    g->offsets = g->col = g->weights = nullptr;
    g->V = 0;
    g->E = 0;
}

dpg_status dpg_write_dimacs9(const char* path, int32_t V, int64_t E, const int32_t* src,
                             const int32_t* dst, const int32_t* w, int32_t source) {
    if (!path || V < 0 || E < 0 || (E > 0 && (!src || !dst || !w)))
        return set_error(DPG_ERR_INVALID_ARG, "dpg_write_dimacs9: bad argument");
    FILE* fp = fopen(path, "w");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot create ") + path);
    FileCloser closer{fp};
    fprintf(fp, "c dpg synthetic graph\np sp %d %" PRId64 "\n", V, E);
    if (source >= 0) fprintf(fp, "s %d\n", source + 1);
    for (int64_t e = 0; e < E; ++e) fprintf(fp, "a %d %d %d\n", src[e] + 1, dst[e] + 1, w[e]);
    if (ferror(fp)) return set_error(DPG_ERR_IO, "write failed");
    return DPG_OK;
}

dpg_status dpg_write_cost(const char* path, int32_t V, int32_t source, const int32_t* dist) {
    if (!path || V < 0 || (V > 0 && !dist)) return set_error(DPG_ERR_INVALID_ARG, "dpg_write_cost: bad argument");
    FILE* fp = fopen(path, "w");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot create ") + path);
    FileCloser closer{fp};
    for (int32_t i = 0; i < V; ++i) fprintf(fp, "From Node %d -> %d is %d\n", source + 1, i + 1, dist[i]);
    return ferror(fp) ? set_error(DPG_ERR_IO, "write failed") : DPG_OK;
}

dpg_status dpg_write_level(const char* path, int32_t V, const int32_t* level) {
    if (!path || V < 0 || (V > 0 && !level)) return set_error(DPG_ERR_INVALID_ARG, "dpg_write_level: bad argument");
    FILE* fp = fopen(path, "w");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot create ") + path);
    FileCloser closer{fp};
    for (int32_t i = 0; i < V; ++i) fprintf(fp, "Node %d is in level %d\n", i + 1, level[i]);
    return ferror(fp) ? set_error(DPG_ERR_IO, "write failed") : DPG_OK;
}

dpg_status dpg_write_rank(const char* path, int32_t V, const float* rank) {
    if (!path || V < 0 || (V > 0 && !rank)) return set_error(DPG_ERR_INVALID_ARG, "dpg_write_rank: bad argument");
    FILE* fp = fopen(path, "w");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot create ") + path);
    FileCloser closer{fp};
    for (int32_t i = 0; i < V; ++i) fprintf(fp, "Node %d: %0.6lf\n", i + 1, static_cast<double>(rank[i]));
    return ferror(fp) ? set_error(DPG_ERR_IO, "write failed") : DPG_OK;
}

dpg_status dpg_write_color(const char* path, int32_t V, const int32_t* color) {
    if (!path || V < 0 || (V > 0 && !color)) return set_error(DPG_ERR_INVALID_ARG, "dpg_write_color: bad argument");
    FILE* fp = fopen(path, "w");
    if (!fp) return set_error(DPG_ERR_IO, std::string("cannot create ") + path);
    FileCloser closer{fp};
    for (int32_t i = 0; i < V; ++i) fprintf(fp, "Node %d: %d\n", i + 1, color[i]);
    return ferror(fp) ? set_error(DPG_ERR_IO, "write failed") : DPG_OK;
}

dpg_status dpg_rmat_arcs(int32_t scale, int32_t V, int64_t E, uint64_t seed, double a, double b,
                         double c, int32_t wmin, int32_t wmax, int32_t permute, int32_t* src,
                         int32_t* dst, int32_t* w) {
    if (scale < 1 || scale > 30 || V < 1 || V > (1 << scale) || E < 0 || (E > 0 && (!src || !dst)))
        return set_error(DPG_ERR_INVALID_ARG, "dpg_rmat_arcs: bad scale / sizes");
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return set_error(DPG_ERR_INVALID_ARG, "dpg_rmat_arcs: bad probabilities");
    if (w && (wmin > wmax)) return set_error(DPG_ERR_INVALID_ARG, "dpg_rmat_arcs: wmin > wmax");
    if (V <= (1 << scale) / 2 && scale > 1) return set_error(DPG_ERR_INVALID_ARG, "dpg_rmat_arcs: scale larger than needed for V");
    // 16-bit thresholds per recursion level; one 64-bit draw feeds four levels.
    const uint32_t ta = static_cast<uint32_t>(llround(a * 65536.0));
    const uint32_t tab = static_cast<uint32_t>(llround((a + b) * 65536.0));
    const uint32_t tabc = static_cast<uint32_t>(llround((a + b + c) * 65536.0));
    const uint64_t wspan = w ? static_cast<uint64_t>(static_cast<int64_t>(wmax) - wmin + 1) : 1;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t e = 0; e < E; ++e) {
        uint32_t u = 0, v = 0;
        for (uint64_t attempt = 0;; ++attempt) {
            u = 0;
            v = 0;
            uint64_t bits = 0;
            for (int lvl = 0; lvl < scale; ++lvl) {
                if ((lvl & 3) == 0) bits = draw(seed, static_cast<uint64_t>(e), attempt * 64 + static_cast<uint64_t>(lvl >> 2));
                const uint32_t r = static_cast<uint32_t>(bits & 0xFFFFu);
                bits >>= 16;
                const uint32_t sb = (r >= tab) ? 1u : 0u;                     // quadrants c,d: source bit 1
                const uint32_t db = (r >= ta && r < tab) || (r >= tabc) ? 1u : 0u;  // quadrants b,d: dest bit 1
                u = (u << 1) | sb;
                v = (v << 1) | db;
            }
            if (permute) {
                u = permute_id(u, scale, seed);
                v = permute_id(v, scale, seed);
            }
            if (static_cast<int64_t>(u) < V && static_cast<int64_t>(v) < V) break;
            if (attempt > 4096) {
                bad = 1;
                break;
            }
        }
        src[e] = static_cast<int32_t>(u);
        dst[e] = static_cast<int32_t>(v);
        if (w) w[e] = wmin + static_cast<int32_t>(draw(seed, static_cast<uint64_t>(e), 0xFFFFFFFFull) % wspan);
    }
    if (bad) return set_error(DPG_ERR_CAPACITY, "dpg_rmat_arcs: rejection sampling did not converge");
    return DPG_OK;
}

dpg_status dpg_grid_arcs(int32_t rows, int32_t cols, uint64_t seed, int32_t wmin, int32_t wmax,
                         int32_t* src, int32_t* dst, int32_t* w) {
    if (rows < 1 || cols < 1 || static_cast<int64_t>(rows) * cols > INT32_MAX || wmin > wmax)
        return set_error(DPG_ERR_INVALID_ARG, "dpg_grid_arcs: bad sizes");
    const int64_t horiz = static_cast<int64_t>(rows) * (cols - 1);
    const int64_t vert = static_cast<int64_t>(cols) * (rows - 1);
    if (2 * (horiz + vert) > INT32_MAX) return set_error(DPG_ERR_CAPACITY, "dpg_grid_arcs: too many arcs");
    if ((horiz + vert) > 0 && (!src || !dst)) return set_error(DPG_ERR_INVALID_ARG, "dpg_grid_arcs: null output");
    const uint64_t wspan = static_cast<uint64_t>(static_cast<int64_t>(wmax) - wmin + 1);
    // Undirected edge k (horizontal ones first, row-major; then vertical ones, row-major) becomes
    // arcs 2k (u->v) and 2k+1 (v->u) with one shared weight, like the paired arcs of a road .gr file.
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < horiz + vert; ++k) {
        int64_t u, v;
        if (k < horiz) {
            const int64_t r = k / (cols - 1), cc = k % (cols - 1);
            u = r * cols + cc;
            v = u + 1;
        } else {
            const int64_t kk = k - horiz;
            const int64_t r = kk / cols, cc = kk % cols;
            u = r * cols + cc;
            v = u + cols;
        }
        const int32_t wt = wmin + static_cast<int32_t>(draw(seed, static_cast<uint64_t>(k), 0x5EEDull) % wspan);
        src[2 * k] = static_cast<int32_t>(u);
        dst[2 * k] = static_cast<int32_t>(v);
        src[2 * k + 1] = static_cast<int32_t>(v);
        dst[2 * k + 1] = static_cast<int32_t>(u);
        if (w) {
            w[2 * k] = wt;
            w[2 * k + 1] = wt;
        }
    }
    return DPG_OK;
}

// Longest-processing-time-first: units by cost descending (ties: lower index first), each to the
// part with the smallest load so far (ties: lower part). Deterministic, so every rank computes the
// same owners on its own.
dpg_status dpg_partition_lpt(int32_t n, const int64_t* cost, int32_t parts, int32_t* owner, int64_t* load) {
    if (n < 0 || parts < 1 || (n > 0 && (!cost || !owner)))
        return set_error(DPG_ERR_INVALID_ARG, "need n >= 0, parts >= 1, costs and owners");
    for (int32_t i = 0; i < n; ++i)
        if (cost[i] < 0) return set_error(DPG_ERR_INVALID_ARG, "costs must be >= 0");
    std::vector<int32_t> order(static_cast<size_t>(n));
    for (int32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
    std::vector<int64_t> ld(static_cast<size_t>(parts), 0);
    for (int32_t i : order) {
        int32_t best = 0;
        for (int32_t p = 1; p < parts; ++p)
            if (ld[p] < ld[best]) best = p;
        owner[i] = best;
        ld[best] += cost[i];
    }
    if (load)
        for (int32_t p = 0; p < parts; ++p) load[p] = ld[p];
    return DPG_OK;
}

}  // extern "C"
