// sgfim_tensorfim <fimi> <rel_thr> -- drop-in for CoParaCG_{baseline,bmma}.exe.
//
// Process contract of the reference (code/pipeline/engine_adapter.py:70-100,
// kernel_bitmap.cu:796-911): reads the FIMI file, mines MFIs at relative
// threshold rel_thr, writes "<fimi>-<rel_thr %f>=Results.txt" next to the
// dataset and prints computation_time(s) / total_time(s).  Threshold rules
// follow kernel_bmma.cu:1189-1233: an extension needs count >= transNum *
// rel_thr (double), a root item needs count / transNum > rel_thr (strict),
// id 0 is never a candidate.  Exit code 0 on success (the reference returns 1).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "sgfim.h"

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <fimi> <rel_thr>\n", argv[0]);
        return 2;
    }
    const char *path = argv[1];
    const double thr = atof(argv[2]);
    auto t0 = std::chrono::steady_clock::now();
    sgfim_config cfg{};
    cfg.flags = SGFIM_F_IGNORE_ID0;
    sgfim_handle *h = nullptr;
    int rc = sgfim_open(&cfg, &h);
    if (rc) {
        fprintf(stderr, "sgfim_open failed (%d)\n", rc);
        return 3;
    }
    if ((rc = sgfim_load_fimi(h, path)) != SGFIM_OK) {
        fprintf(stderr, "%s open failed! (%s)\n", path, sgfim_last_error(h));
        sgfim_close(h);
        return 1;
    }
    auto t1 = std::chrono::steady_clock::now();
    sgfim_dataset_info info{};
    sgfim_dataset_info_get(h, &info);
    const double n = (double)info.n_txn;
    const double fthr = n * thr;
    uint32_t min_count = (uint32_t)std::max(1.0, std::ceil(fthr));
    // smallest count c with c / n > thr (the strict root rule)
    uint64_t root_min = (uint64_t)std::max(0.0, std::floor(fthr));
    while (n > 0 && (double)root_min / n <= thr) ++root_min;
    std::vector<uint32_t> counts(info.n_ids);
    sgfim_item_counts(h, counts.data(), info.n_ids);
    uint32_t dim_red = 0;
    for (uint32_t id = 0; id < info.n_ids; ++id)
        if (n > 0 && (double)counts[id] / n > thr) ++dim_red;
    sgfim_mine_params p{};
    p.min_count = min_count;
    p.root_rule = SGFIM_ROOTS_MINCOUNT;
    p.root_min_count = (uint32_t)std::min<uint64_t>(root_min, 0xffffffffu);
    sgfim_result *res = nullptr;
    rc = sgfim_mine(h, &p, &res);
    if (rc) {
        fprintf(stderr, "mining failed: %s\n", sgfim_last_error(h));
        sgfim_close(h);
        return 1;
    }
    auto t2 = std::chrono::steady_clock::now();
    const double pre = std::chrono::duration<double>(t1 - t0).count();
    const double comp = std::chrono::duration<double>(t2 - t1).count();
    char thr_s[64];
    snprintf(thr_s, sizeof thr_s, "%f", thr);
    const std::string out = std::string(path) + "-" + thr_s + "=Results.txt";
    sgfim_tf_meta meta{};
    meta.trans_set_file = path;
    meta.support_threshold = thr;
    meta.computation_time_s = comp;
    meta.preprocessing_time_s = pre;
    meta.dimension_reduced = dim_red;
    rc = sgfim_write_tensorfim(h, res, &meta, out.c_str());
    printf("MFIsNumber: %llu\n", (unsigned long long)res->n_sets);
    printf("preprocessing_time(s): %g\ncomputation_time(s): %g\ntotal_time(s): %g\n", pre, comp, pre + comp);
    sgfim_result_free(res);
    sgfim_close(h);
    return rc ? 1 : 0;
}
