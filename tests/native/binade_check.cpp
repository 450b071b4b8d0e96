// Checks the binade-wise parallel formulation of the reference's serial double
// prefix sum s_m = fl64(s_{m-1} + w_m) (novel_resampling.h:53-56, weights >= 0)
// that the systematic resampler's exact fallback uses on the device, against
// plain serial double additions, on random float weights with zeros, tiny and
// huge values and constructed round-to-even ties.
//
// Within one binade [2^b, 2^(b+1)) of the running sum every result is a
// multiple of u = 2^(b-52), so s_k = s_{k-1} + r_k u with
// r_k = floor(w_k / u) + [frac > 1/2] independent of s, except at ties
// (frac == 1/2) and where the sum leaves the binade; those "events" are
// resolved by one ordinary double addition.  Here the chunk logic is serial,
// but every quantity is computed as the device computes it (prefix sums of r
// over a chunk, first event position).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

static double pow2(int k) { return std::ldexp(1.0, k); }
static int binade(double s) { int e; std::frexp(s, &e); return e - 1; }   // s in [2^b, 2^(b+1))

static long g_ties = 0, g_exits = 0;

static void binade_sums(const float* w, size_t M, double* out, size_t chunk)
{
    double s = 0.0;
    for (size_t c0 = 0; c0 < M; c0 += chunk) {
        const size_t c1 = std::min(M, c0 + chunk);
        size_t pos = c0;
        while (pos < c1) {
            if (s == 0.0) {   // leading zero weights keep s = 0; the first positive one is s exactly
                size_t z = pos;
                while (z < c1 && w[z] == 0.0f) out[z++] = 0.0;
                if (z < c1) {
                    s = (double)w[z];
                    out[z] = s;
                    ++z;
                }
                pos = z;
                continue;
            }
            const int b = binade(s);
            const double u = pow2(b - 52), uinv = pow2(52 - b), top = pow2(b + 1);
            const uint64_t P0 = (uint64_t)(s * uinv);   // exact, in [2^52, 2^53)
            const uint64_t LIM = 1ull << 53;
            // per element: q, the increment r (ties: +1 when the running sum before the
            // tie plus q is odd -- round half to even; the sum after a tie is always
            // even, so the parity before a tie is that of the start or the last tie
            // XOR the low bits of the increments since: a segmented XOR scan), and
            // whether the exact sum leaves the binade (then one double addition)
            size_t first_event = c1;
            uint64_t run = 0;
            uint32_t par = (uint32_t)(P0 & 1);   // parity of the running sum so far
            std::vector<uint64_t> incl(c1 - pos);
            for (size_t k = pos; k < c1; ++k) {
                const double wd = (double)w[k];
                uint64_t r = 0, q = 0;
                bool ev = false;
                if (wd >= top) {
                    ev = true;
                } else {
                    const double t = wd * uinv;   // exact scaling
                    q = (uint64_t)t;
                    const double f = t - (double)q;
                    if (f == 0.5) {
                        ++g_ties;
                        r = q + ((par ^ (uint32_t)(q & 1)) & 1);
                        par = 0;
                    } else {
                        r = q + (f > 0.5 ? 1 : 0);
                        par ^= (uint32_t)(r & 1);
                    }
                }
                if (!ev && P0 + run + q >= LIM) {   // the exact sum leaves the binade
                    ev = true;
                    ++g_exits;
                }
                if (ev && first_event == c1) first_event = k;
                run += r > LIM ? LIM : r;
                incl[k - pos] = run;
            }
            for (size_t k = pos; k < first_event; ++k) out[k] = (double)(P0 + incl[k - pos]) * u;
            if (first_event < c1) {
                const double before = first_event > pos ? (double)(P0 + incl[first_event - 1 - pos]) * u : s;
                s = before + (double)w[first_event];   // one ordinary double addition
                out[first_event] = s;
                pos = first_event + 1;
            } else {
                s = (double)(P0 + incl[c1 - 1 - pos]) * u;
                pos = c1;
            }
        }
    }
}

int main()
{
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long bad = 0, cases = 0;
    for (int trial = 0; trial < 300; ++trial) {
        const size_t M = 1 + rng() % 20000;
        std::vector<float> w(M);
        const int kind = trial % 5;
        for (size_t i = 0; i < M; ++i) {
            double x = U(rng);
            if (kind == 0) x = std::pow(x, 8.0) * 1e-6;                 // tiny
            else if (kind == 1) x = (rng() % 4 == 0) ? 0.0 : x * x * 1e-7;
            else if (kind == 2) x = std::exp(-40.0 * x);                // huge range
            else if (kind == 3) x = (rng() % 100 == 0) ? x : x * 1e-12;
            else x = 1.0 / (double)M;
            w[i] = (float)x;
        }
        if (kind == 4) {   // plant ties: weights exactly (k + 1/2) ulps of the running sum
            double s = 0.0;
            for (size_t i = 0; i < M; ++i) {
                if (i > 10 && rng() % 50 == 0 && s > 0.0) {
                    const double u = pow2(binade(s) - 52);
                    w[i] = (float)((double)(1 + rng() % 1000) * u + 0.5 * u);   // exact in float
                }
                s += (double)w[i];
            }
        }
        std::vector<double> ref(M), got(M);
        double s = 0.0;
        for (size_t i = 0; i < M; ++i) {
            s += (double)w[i];
            ref[i] = s;
        }
        binade_sums(w.data(), M, got.data(), 1 + rng() % 4096);
        ++cases;
        if (std::memcmp(ref.data(), got.data(), sizeof(double) * M) != 0) {
            size_t k = 0;
            while (ref[k] == got[k]) ++k;
            if (bad < 5) std::printf("mismatch trial %d kind %d M %zu at %zu: %.17g vs %.17g\n", trial, kind, M, k,
                                     ref[k], got[k]);
            ++bad;
        }
    }
    std::printf("binade sums: %ld cases, %ld mismatches, %ld ties, %ld binade exits\n", cases, bad, g_ties, g_exits);
    return bad ? 1 : 0;
}
