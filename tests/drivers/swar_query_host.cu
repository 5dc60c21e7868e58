// Runs the SQF one-byte-slot query state machine (sqf_query_b1, the device
// code's own function, compiled for the host) over a table and a list of
// fingerprints read from files, and writes the results.  Used by the CPU
// tests to check the byte-lane SWAR walk against the oracle without a GPU.
//   swar_query_host <table.bin> <fps.bin> <q> <r> <nslots> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../gpuquotientfilters_gb300/csrc/sqf_lookup.cuh"

static std::vector<unsigned char> slurp(const char *path)
{
    std::vector<unsigned char> b;
    FILE *f = std::fopen(path, "rb");
    if (!f) return b;
    unsigned char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + k);
    std::fclose(f);
    return b;
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s table fps q r nslots out\n", argv[0]);
        return 2;
    }
    std::vector<unsigned char> tab = slurp(argv[1]), fpb = slurp(argv[2]);
    const uint32_t q = (uint32_t)std::atoi(argv[3]), r = (uint32_t)std::atoi(argv[4]);
    const uint32_t nslots = (uint32_t)std::strtoul(argv[5], nullptr, 10);
    if (tab.size() < nslots || fpb.size() % 4) return 3;
    // keep the word loads inside the buffer: the byte-wise tail path covers the rest
    gqf::TableView v{tab.data(), q, r, nslots, (uint32_t)tab.size(), (uint32_t)(tab.size() / 8)};
    const size_t n = fpb.size() / 4;
    const uint32_t *fps = reinterpret_cast<const uint32_t *>(fpb.data());
    // with SWAR_SUMMARY set, each query gets its home word's pending-run
    // summary byte (the recurrence the summary kernel scans)
    const bool use_sum = std::getenv("SWAR_SUMMARY") != nullptr;
    std::vector<int> P;
    if (use_sum) {
        const uint32_t nwords = (nslots + 7) / 8;
        P.resize(nwords);
        int p = 0;
        for (uint32_t w = 0; w < nwords; w++) {
            P[w] = p < 0 || p > 254 ? 255 : p;
            p = gqf::pend_apply(gqf::pend_word(gqf::ld_word(v, w)), p);
        }
    }
    std::vector<uint32_t> out(n);
    for (size_t i = 0; i < n; i++) {
        const uint32_t fq = (fps[i] >> r) & ((1u << q) - 1u), fr = fps[i] & ((1u << r) - 1u);
        out[i] = gqf::sqf_query_b1(v, fq, fr, gqf::ld_word(v, fq >> 3), use_sum ? P[fq >> 3] : -1);
    }
    FILE *f = std::fopen(argv[6], "wb");
    if (!f) return 4;
    std::fwrite(out.data(), 4, n, f);
    std::fclose(f);
    return 0;
}
