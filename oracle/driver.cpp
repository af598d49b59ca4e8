// Oracle (test infrastructure only): the chunk driver of src/main.rs, shared by the
// command line (main.cpp) and the in-memory entry points (capi.cpp ora_map_batch,
// ora_map_interleaved), and the pairing of interleaved input (src/io/reads.rs:68-113).
// Chunks are records until the nucleotide count exceeds chunk_size
// (src/main.rs:591-604); each gets a fresh Rng::with_seed(0) and
// InsertSizeDistribution (:878-879); outputs are kept per chunk, in chunk order
// (:653-667).  Chunks run on `threads` threads.
#include <atomic>
#include <thread>

#include "oracle.hpp"

namespace oracle {

std::vector<std::pair<size_t, size_t>> chunk_ranges(const std::vector<SequenceRecord>& r1,
                                                    const std::vector<SequenceRecord>* r2, size_t chunk_size,
                                                    const std::vector<uint8_t>* has_mate) {
    size_t n = r2 ? std::min(r1.size(), r2->size()) : r1.size();
    std::vector<std::pair<size_t, size_t>> chunks;
    for (size_t i = 0; i < n;) {
        size_t nt = 0, j = i;
        while (j < n) {
            const bool pe = r2 && (!has_mate || (*has_mate)[j]);
            nt += r1[j].seq.size() + (pe ? (*r2)[j].seq.size() : 0);
            j++;
            if (nt > chunk_size) break;
        }
        chunks.emplace_back(i, j);
        i = j;
    }
    return chunks;
}

void pair_interleaved(std::vector<SequenceRecord>&& records, std::vector<SequenceRecord>& r1,
                      std::vector<SequenceRecord>& r2, std::vector<uint8_t>& has_mate) {
    r1.clear();
    r2.clear();
    has_mate.clear();
    for (size_t i = 0; i < records.size();) {
        const bool pair = i + 1 < records.size() && records[i].name == records[i + 1].name;
        r1.push_back(std::move(records[i]));
        if (pair) r2.push_back(std::move(records[i + 1]));
        else r2.emplace_back();
        has_mate.push_back(pair ? 1 : 0);
        i += pair ? 2 : 1;
    }
}

std::vector<std::string> map_records(const Context& ctx, const std::vector<SequenceRecord>& r1,
                                     const std::vector<SequenceRecord>* r2, MapMode mode, size_t threads,
                                     size_t chunk_size, std::vector<double>* abundances,
                                     const std::vector<uint8_t>* has_mate) {
    auto chunks = chunk_ranges(r1, r2, chunk_size, has_mate);
    std::vector<std::string> outs(chunks.size());
    size_t nt = std::max<size_t>(threads, 1);
    size_t n_refs = ctx.refs->size();
    std::vector<std::vector<double>> ab(mode == MapMode::Abundance ? nt : 0, std::vector<double>(n_refs, 0.0));
    std::atomic<size_t> next{0};
    auto worker = [&](size_t tid) {
        for (;;) {
            size_t c = next.fetch_add(1);
            if (c >= chunks.size()) break;
            Rng rng(0);
            InsertSizeDistribution isd;
            std::string& out = outs[c];
            for (size_t i = chunks[c].first; i < chunks[c].second; i++) {
                Details d;
                // a record with a mate is a pair (src/main.rs:886-985 matches on r2)
                const bool pe = r2 && (!has_mate || (*has_mate)[i]);
                if (mode == MapMode::Abundance) {
                    if (pe) abundances_paired_end_read(r1[i], (*r2)[i], ctx, ab[tid], isd, rng);
                    else abundances_single_end_read(r1[i], ctx, ab[tid], rng);
                } else if (mode == MapMode::Paf) {
                    out += pe ? map_paired_end_read(r1[i], (*r2)[i], ctx, isd, rng, d) : map_single_end_read(r1[i], ctx, rng, d);
                } else {
                    out += pe ? align_paired_end_read(r1[i], (*r2)[i], ctx, isd, rng, d)
                              : align_single_end_read(r1[i], ctx, rng, d);
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; t++) th.emplace_back(worker, t);
    for (auto& t : th) t.join();
    if (abundances) {
        abundances->assign(n_refs, 0.0);
        for (size_t t = 0; t < ab.size(); t++)
            for (size_t i = 0; i < n_refs; i++) (*abundances)[i] += ab[t][i];
    }
    return outs;
}

}  // namespace oracle
