// Seeded synthetic alignment workloads (DNA and protein pairs).
//
// Stands in for the reference's test sets, whose DNA inputs and protein
// references are not shipped with it.  A pair is a reference (contig, "A")
// and a query (read, "B").  Queries are either unrelated random sequences or
// mutated copies of a random substring of their reference:
//   * DNA: per-position substitution (uniform over the other three bases) and
//     indel events (insertion or deletion with equal odds, length geometric);
//   * protein: per-position substitution drawn from the BLOSUM62 target
//     distribution P(b | a) ~ p_b * 2^(s_ab / 2), with the substitution rate
//     solved so that the expected identity hits a requested value, plus indels.
// Lengths are uniform on [min, max] or log-normal (median, sigma) clipped to
// [min, max].  A workload is a mixture of up to four such components.
//
// The PRNG is xoshiro256** seeded through splitmix64: the same seed gives the
// same bytes on any host.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbsw_synth.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int k = 0; k < 4; ++k) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            s[k] = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // integer in [lo, hi]
    int64_t range(int64_t lo, int64_t hi) {
        uint64_t span = (uint64_t)(hi - lo + 1);
        return lo + (int64_t)(next() % span);
    }
    double normal() {
        double u1 = uniform();
        double u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
    // geometric on {1, 2, ...} with the given mean (>= 1)
    int geometric(double mean) {
        double p = 1.0 / mean;
        int k = 1;
        while (uniform() >= p && k < 1000000) ++k;
        return k;
    }
};

const char kDna[4] = {'A', 'C', 'G', 'T'};
const char kAA[20] = {'A', 'R', 'N', 'D', 'C', 'Q', 'E', 'G', 'H', 'I',
                      'L', 'K', 'M', 'F', 'P', 'S', 'T', 'W', 'Y', 'V'};

// Cumulative tables for drawing residues.
struct AATables {
    double bg_cdf[20];
    double cond_cdf[20][20];  // P(b | a) cumulative over b
    double self_avg;          // sum_a p_a P(a | a)
};

bool build_aa_tables(const gbsw_synth_params* p, AATables* t) {
    double bg[20];
    double tot = 0;
    for (int k = 0; k < 20; ++k) {
        bg[k] = p->aa_background[k] > 0 ? p->aa_background[k] : 0;
        tot += bg[k];
    }
    if (tot <= 0) return false;
    double acc = 0;
    for (int k = 0; k < 20; ++k) {
        bg[k] /= tot;
        acc += bg[k];
        t->bg_cdf[k] = acc;
    }
    t->bg_cdf[19] = 1.0;
    t->self_avg = 0;
    for (int a = 0; a < 20; ++a) {
        double w[20];
        double sum = 0;
        for (int b = 0; b < 20; ++b) {
            // p->aa_matrix is 20x20 in kAA order (the first 20 residues of the
            // 24-letter order)
            w[b] = bg[b] * std::pow(2.0, p->aa_matrix[a * 20 + b] / 2.0);
            sum += w[b];
        }
        double c = 0;
        for (int b = 0; b < 20; ++b) {
            c += w[b] / sum;
            t->cond_cdf[a][b] = c;
        }
        t->cond_cdf[a][19] = 1.0;
        t->self_avg += bg[a] * (w[a] / sum);
    }
    return true;
}

int draw_cdf(Rng& r, const double* cdf, int n) {
    double u = r.uniform();
    for (int k = 0; k < n; ++k)
        if (u < cdf[k]) return k;
    return n - 1;
}

int draw_len(Rng& r, const gbsw_synth_len& L) {
    int v;
    if (L.dist == GBSW_SYNTH_LOGNORMAL) {
        double x = L.median * std::exp(L.sigma * r.normal());
        v = (int)std::lround(x);
    } else {
        v = (int)r.range(L.min, L.max);
    }
    if (v < L.min) v = L.min;
    if (v > L.max) v = L.max;
    return v;
}

char random_residue(Rng& r, int alphabet, const AATables* t) {
    if (alphabet == GBSW_SYNTH_DNA) return kDna[r.next() & 3];
    return kAA[draw_cdf(r, t->bg_cdf, 20)];
}

int aa_index(char c) {
    for (int k = 0; k < 20; ++k)
        if (kAA[k] == c) return k;
    return 0;
}

char substitute(Rng& r, char c, int alphabet, const AATables* t) {
    if (alphabet == GBSW_SYNTH_DNA) {
        int idx = 0;
        for (int k = 0; k < 4; ++k)
            if (kDna[k] == c) idx = k;
        int other = (int)(r.next() % 3);
        return kDna[(idx + 1 + other) & 3];
    }
    return kAA[draw_cdf(r, t->cond_cdf[aa_index(c)], 20)];
}

void mutate(Rng& r, const std::string& src, const gbsw_synth_component& c, double sub_rate,
            const AATables* t, std::string* out) {
    out->clear();
    out->reserve(src.size() + 16);
    size_t k = 0;
    while (k < src.size()) {
        if (c.indel_rate > 0 && r.uniform() < c.indel_rate) {
            int len = r.geometric(c.indel_mean > 1 ? c.indel_mean : 1.0);
            if (r.next() & 1) {  // insertion of random residues
                for (int q = 0; q < len; ++q) out->push_back(random_residue(r, c.alphabet, t));
            } else {  // deletion
                k += (size_t)len;
                continue;
            }
        }
        char ch = src[k];
        if (sub_rate > 0 && r.uniform() < sub_rate) ch = substitute(r, ch, c.alphabet, t);
        out->push_back(ch);
        ++k;
    }
    if (out->empty()) out->push_back(src.empty() ? random_residue(r, c.alphabet, t) : src[0]);
}

}  // namespace

extern "C" int gbsw_synth_generate(const gbsw_synth_params* p, int64_t n, uint64_t seed,
                                   gbsw_synth_batch* out) {
    if (!p || !out || n < 0 || p->ncomponents < 1 || p->ncomponents > GBSW_SYNTH_MAX_COMPONENTS)
        return -1;
    std::memset(out, 0, sizeof(*out));
    AATables tables;
    bool have_tables = build_aa_tables(p, &tables);
    double wsum = 0;
    for (int c = 0; c < p->ncomponents; ++c) {
        const gbsw_synth_component& comp = p->components[c];
        if (comp.weight < 0) return -1;
        if (comp.alphabet == GBSW_SYNTH_PROTEIN && !have_tables) return -1;
        if (comp.ref_len.min < 1 || comp.ref_len.max < comp.ref_len.min) return -1;
        if (comp.query_len.min < 1 || comp.query_len.max < comp.query_len.min) return -1;
        wsum += comp.weight;
    }
    if (wsum <= 0) return -1;

    Rng rng(seed);
    std::vector<std::string> refs((size_t)n), qs((size_t)n);
    std::vector<int> comp_of((size_t)n);
    std::string sub, tmp;
    int64_t ref_total = 0, q_total = 0;
    for (int64_t k = 0; k < n; ++k) {
        double u = rng.uniform() * wsum;
        int ci = 0;
        double acc = 0;
        for (; ci < p->ncomponents - 1; ++ci) {
            acc += p->components[ci].weight;
            if (u < acc) break;
        }
        const gbsw_synth_component& c = p->components[ci];
        comp_of[(size_t)k] = ci;
        int rl = draw_len(rng, c.ref_len);
        std::string& R = refs[(size_t)k];
        R.resize((size_t)rl);
        for (int q = 0; q < rl; ++q) R[(size_t)q] = random_residue(rng, c.alphabet, &tables);
        std::string& Q = qs[(size_t)k];
        if (rng.uniform() < c.related_fraction) {
            int ql = c.query_from_ref_length ? rl : draw_len(rng, c.query_len);
            if (ql > rl) ql = rl;
            int start = (int)rng.range(0, rl - ql);
            sub.assign(R, (size_t)start, (size_t)ql);
            double sub_rate = c.substitution_rate;
            if (c.alphabet == GBSW_SYNTH_PROTEIN && c.target_identity > 0) {
                // identity = (1 - r) + r * self_avg  ->  r = (1 - id) / (1 - self_avg)
                sub_rate = (1.0 - c.target_identity) / (1.0 - tables.self_avg);
                if (sub_rate > 1) sub_rate = 1;
                if (sub_rate < 0) sub_rate = 0;
            }
            mutate(rng, sub, c, sub_rate, &tables, &Q);
        } else {
            int ql = draw_len(rng, c.query_len);
            Q.resize((size_t)ql);
            for (int q = 0; q < ql; ++q) Q[(size_t)q] = random_residue(rng, c.alphabet, &tables);
        }
        ref_total += (int64_t)R.size();
        q_total += (int64_t)Q.size();
    }

    out->n = n;
    out->ref_total = ref_total;
    out->query_total = q_total;
    out->ref = (char*)std::malloc((size_t)ref_total + 1);
    out->query = (char*)std::malloc((size_t)q_total + 1);
    out->ref_off = (int64_t*)std::malloc(sizeof(int64_t) * (size_t)(n + 1));
    out->query_off = (int64_t*)std::malloc(sizeof(int64_t) * (size_t)(n + 1));
    out->component = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)(n + 1));
    if (!out->ref || !out->query || !out->ref_off || !out->query_off || !out->component) {
        gbsw_synth_free(out);
        return -2;
    }
    int64_t ra = 0, qa = 0;
    for (int64_t k = 0; k < n; ++k) {
        out->ref_off[k] = ra;
        out->query_off[k] = qa;
        out->component[k] = comp_of[(size_t)k];
        std::memcpy(out->ref + ra, refs[(size_t)k].data(), refs[(size_t)k].size());
        std::memcpy(out->query + qa, qs[(size_t)k].data(), qs[(size_t)k].size());
        ra += (int64_t)refs[(size_t)k].size();
        qa += (int64_t)qs[(size_t)k].size();
    }
    out->ref_off[n] = ra;
    out->query_off[n] = qa;
    return 0;
}

extern "C" void gbsw_synth_free(gbsw_synth_batch* b) {
    if (!b) return;
    std::free(b->ref);
    std::free(b->query);
    std::free(b->ref_off);
    std::free(b->query_off);
    std::free(b->component);
    std::memset(b, 0, sizeof(*b));
}
