// sgfim_anytime <fimi> <upto_stage> -- drop-in for AnytimeMining.exe.
//
// Stage semantics of the reference (AnytimeMining/kernel.cu:798-915): ids are
// ordered by occurrence count, descending and stable (ties: ascending id),
// over ids 0..itemIDmax; stage k mines at threshold = the k-th count of that
// order with the first k ids as roots; each stage's pool is sorted by
// frequency and all stages are written to "<fimi>-<upto_stage>-stages=Results.txt"
// once every stage has finished.  upto_stage greater than the number of
// distinct ids prints the reference's message and writes nothing.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <string>
#include <vector>

#include "sgfim.h"

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <fimi> <upto_stage>\n", argv[0]);
        return 2;
    }
    const char *path = argv[1];
    const int upto = atoi(argv[2]);
    auto t0 = std::chrono::steady_clock::now();
    sgfim_config cfg{};
    cfg.flags = SGFIM_F_IGNORE_ID0;
    sgfim_handle *h = nullptr;
    if (sgfim_open(&cfg, &h)) {
        fprintf(stderr, "sgfim_open failed\n");
        return 3;
    }
    if (sgfim_load_fimi(h, path)) {
        fprintf(stderr, "%s open failed! (%s)\n", path, sgfim_last_error(h));
        sgfim_close(h);
        return 1;
    }
    sgfim_dataset_info info{};
    sgfim_dataset_info_get(h, &info);
    if (upto < 1 || (uint32_t)upto > info.n_present) {
        printf("Up to the stage number being greater than the dimension !\n");
        sgfim_close(h);
        return 0;
    }
    std::vector<uint32_t> counts(info.n_ids);
    sgfim_item_counts(h, counts.data(), info.n_ids);
    std::vector<uint32_t> order(info.n_ids);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return counts[a] > counts[b]; });
    auto t1 = std::chrono::steady_clock::now();
    const double pre = std::chrono::duration<double>(t1 - t0).count();
    std::vector<sgfim_result *> stages(upto, nullptr);
    std::vector<double> rt(upto);
    std::vector<uint32_t> fthr(upto);
    int rc = 0;
    for (int k = 1; k <= upto && rc == 0; ++k) {
        auto s0 = std::chrono::steady_clock::now();
        const uint32_t thr = (uint32_t)k - 1 < order.size() ? counts[order[k - 1]] : 0;
        fthr[k - 1] = thr;
        std::vector<uint32_t> roots(order.begin(), order.begin() + std::min<size_t>(k, order.size()));
        sgfim_mine_params p{};
        p.min_count = std::max<uint32_t>(thr, 1);
        p.root_rule = SGFIM_ROOTS_LIST;
        p.roots = roots.data();
        p.n_roots = (uint32_t)roots.size();
        rc = sgfim_mine(h, &p, &stages[k - 1]);
        rt[k - 1] = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
        if (rc == 0)
            printf("%dth stage MFIsNum: %llu, runtime: %g\n", k, (unsigned long long)stages[k - 1]->n_sets, rt[k - 1]);
    }
    if (rc) {
        fprintf(stderr, "mining failed: %s\n", sgfim_last_error(h));
    } else {
        sgfim_af_meta meta{};
        meta.trans_set_file = path;
        meta.upto_stage = (uint32_t)upto;
        meta.preprocessing_time_s = pre;
        meta.runtime_per_stage_s = rt.data();
        meta.frequency_thr_per_stage = fthr.data();
        const std::string out = std::string(path) + "-" + std::to_string(upto) + "-stages=Results.txt";
        rc = sgfim_write_anyfim(h, stages.data(), &meta, out.c_str());
        double tot = pre;
        for (double v : rt) tot += v;
        printf("preprocessing_time(s): %g\ncomputation_time(s): %g\ntotal_time(s): %g\n", pre, tot - pre, tot);
    }
    for (auto *r : stages) sgfim_result_free(r);
    sgfim_close(h);
    return rc ? 1 : 0;
}
