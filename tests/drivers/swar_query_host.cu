// Runs the SQF one-byte-slot query state machine (sqf_query_b1, the device
// code's own function, compiled for the host) over a table and a list of
// fingerprints read from files, and writes the results.  Used by the CPU
// tests to check the byte-lane SWAR walk against the oracle without a GPU.
// With SWAR_MIRROR set, the queries go through the bit-plane mirror instead
// (mirror_record / mirror_query, the lookup kernel's own functions), falling
// back to sqf_query_b1 where the two-record window does not decide.  With
// SWAR_MIRROR_GROUPS set it checks the build kernel's transposition
// (mirror_groups) against mirror_record over the whole table instead.
//   swar_query_host <table.bin> <fps.bin> <q> <r> <nslots> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../gpuquotientfilters_gb300/csrc/sqf_mirror.cuh"

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
    std::vector<uint32_t> out(n);
    if (std::getenv("SWAR_MIRROR_GROUPS")) {
        // the build kernel's per-thread transposition (mirror_groups) against
        // mirror_record, over every thread range of 31 words (8 groups)
        const uint32_t ng = gqf::mir_groups(nslots);
        size_t bad = 0, checked = 0;
        for (uint32_t t = 0; 8 * t <= ng; t++) {
            uint64_t sw[gqf::MIR_WORDS];
            for (uint32_t i = 0; i < gqf::MIR_WORDS; i++) sw[i] = gqf::ld_word(v, gqf::MIR_WORDS * t + i);
            uint32_t gp[8][8];
            int cnt[8];
            gqf::mirror_groups(sw, gp, cnt);
            for (uint32_t g = 0; g < 8 && 8 * t + g <= ng; g++) {
                uint32_t r[8];
                gqf::mirror_record(tab.data(), (uint32_t)tab.size(), 8 * t + g, 0, r);
                bool ok = cnt[g] == gqf::popc32(r[0]) - gqf::popc32(r[1]);
                for (int w = 0; w < 8; w++) ok = ok && gp[g][w] == r[w];
                bad += ok ? 0 : 1;
                checked++;
            }
        }
        std::fprintf(stderr, "groups checked %zu, differing %zu\n", checked, bad);
        return bad ? 5 : 0;
    }
    if (std::getenv("SWAR_MIRROR")) {
        const uint32_t ng = gqf::mir_groups(nslots);
        std::vector<uint32_t> rec((size_t)(ng + 1) * 8);
        int D = 0;  // pending runs at the group's first slot
        for (uint32_t G = 0; G <= ng; G++) {
            uint32_t r[8];
            gqf::mirror_record(tab.data(), (uint32_t)tab.size(), G, D, r);
            for (int w = 0; w < 8; w++) rec[(size_t)G * 8 + w] = r[w];
            for (uint32_t j = 0; j < gqf::MIR_SLOTS; j++) {
                const size_t sl = (size_t)G * gqf::MIR_SLOTS + j;
                const uint32_t e = sl < tab.size() ? tab[sl] : 0u;
                D += (int)((e >> 2) & 1u) - (int)((e & 7u) != 0 && !((e >> 1) & 1u));
            }
        }
        size_t undecided = 0;
        for (size_t i = 0; i < n; i++) {
            const uint32_t fq = (fps[i] >> r) & ((1u << q) - 1u), fr = fps[i] & ((1u << r) - 1u);
            const uint32_t G = fq / gqf::MIR_SLOTS;
            uint32_t r0[8], r1[8];
            for (int w = 0; w < 8; w++) {
                r0[w] = rec[(size_t)G * 8 + w];
                r1[w] = rec[(size_t)(G + 1) * 8 + w];
            }
            uint32_t res = gqf::mirror_query(fq, fr, fq - G * gqf::MIR_SLOTS, r0, r1);
            if (res == gqf::MIRROR_UNDECIDED) {
                undecided++;
                res = gqf::sqf_query_b1(v, fq, fr, gqf::ld_word(v, fq >> 3));
            }
            out[i] = res;
        }
        std::fprintf(stderr, "undecided %zu of %zu\n", undecided, n);
        FILE *f = std::fopen(argv[6], "wb");
        if (!f) return 4;
        std::fwrite(out.data(), 4, n, f);
        std::fclose(f);
        return 0;
    }
    for (size_t i = 0; i < n; i++) {
        const uint32_t fq = (fps[i] >> r) & ((1u << q) - 1u), fr = fps[i] & ((1u << r) - 1u);
        out[i] = gqf::sqf_query_b1(v, fq, fr, gqf::ld_word(v, fq >> 3));
    }
    FILE *f = std::fopen(argv[6], "wb");
    if (!f) return 4;
    std::fwrite(out.data(), 4, n, f);
    std::fclose(f);
    return 0;
}
