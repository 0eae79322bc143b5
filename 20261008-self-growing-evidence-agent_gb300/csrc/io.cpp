// io.cpp -- FIMI parsing and Results.txt writers (host).
//
// parse_fimi_file restates readTransSetFile
// (code/engine_tensorfim/code/engine/src/kernel_bitmap.cu:205-233): the file is
// scanned byte by byte; '\n' ends a transaction (an empty line is an empty
// transaction), a run of digits is an item, '-' followed by digits is dropped,
// every other byte separates; a final line without '\n' counts when it holds
// an item.  The scan is split into line-aligned slices parsed in parallel.
//
// The writers emit the record and section layout that
// engine_adapter.parse_tensorfim_results / parse_anyfim_results
// (code/pipeline/engine_adapter.py:29-33,103-166) read back:
//   "<i>th: <k> { <ids...> }   support: <f>  frequency: <count>"
//   "====================== <k>th stage MFIs Number: <m> ======================"
// with the header fields of kernel_bitmap.cu:651-690 and
// AnytimeMining/kernel.cu:615-659.  Doubles print like a default-formatted
// C++ stream (6 significant digits).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>
#include <vector>

#include "engine.h"

namespace sg {

namespace {

struct Slice {
    std::vector<uint64_t> lens;
    std::vector<uint32_t> items;
    bool overflow = false;
};

// Parse bytes [b, e) which start at a line start; `last` marks the file's final slice.
void parse_slice(const char *b, const char *e, bool last, Slice &out) {
    const char *p = b;
    uint64_t cur = 0;
    bool pending = false;  // current line has content worth keeping at EOF
    while (p < e) {
        const char c = *p;
        if (c == '\n') {
            out.lens.push_back(cur);
            cur = 0;
            pending = false;
            ++p;
            continue;
        }
        if (c >= '0' && c <= '9') {
            uint64_t v = 0;
            while (p < e && *p >= '0' && *p <= '9') {
                v = v * 10 + (uint64_t)(*p - '0');
                if (v > 0xfffffffeull) out.overflow = true;
                ++p;
            }
            out.items.push_back((uint32_t)std::min<uint64_t>(v, 0xfffffffeull));
            ++cur;
            pending = true;
            continue;
        }
        if (c == '-') {
            ++p;
            while (p < e && *p >= '0' && *p <= '9') ++p;
            continue;
        }
        ++p;
    }
    if (last && pending) out.lens.push_back(cur);
    else if (!last && cur) out.lens.push_back(cur);  // cannot happen: slices end after '\n'
}

std::string fmt_double(double v) {
    std::ostringstream os;
    os << v;
    return os.str();
}

}  // namespace

int parse_fimi_file(const char *path, std::vector<uint64_t> &row_ptr, std::vector<uint32_t> &items, std::string &err) {
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        err = std::string("cannot open ") + path;
        return SGFIM_EIO;
    }
    fseek(fp, 0, SEEK_END);
    const long long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    std::vector<char> buf(sz > 0 ? (size_t)sz : 1);
    if (sz > 0 && fread(buf.data(), 1, (size_t)sz, fp) != (size_t)sz) {
        fclose(fp);
        err = std::string("short read on ") + path;
        return SGFIM_EIO;
    }
    fclose(fp);
    const char *data = buf.data();
    const size_t n = sz > 0 ? (size_t)sz : 0;
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < (1u << 20)) nt = 1;
    // line-aligned slice boundaries
    std::vector<size_t> cut{0};
    for (unsigned t = 1; t < nt; ++t) {
        size_t pos = n * t / nt;
        while (pos < n && data[pos - 1] != '\n') ++pos;
        if (pos > cut.back() && pos < n) cut.push_back(pos);
    }
    cut.push_back(n);
    const size_t ns = cut.size() - 1;
    std::vector<Slice> sl(ns);
    std::vector<std::thread> th;
    for (size_t s = 0; s < ns; ++s)
        th.emplace_back([&, s] { parse_slice(data + cut[s], data + cut[s + 1], s + 1 == ns, sl[s]); });
    for (auto &t : th) t.join();
    size_t nrows = 0, nitems = 0;
    for (auto &s : sl) {
        if (s.overflow) {
            err = "item id exceeds 32 bits";
            return SGFIM_EINVAL;
        }
        nrows += s.lens.size();
        nitems += s.items.size();
    }
    row_ptr.assign(nrows + 1, 0);
    items.resize(nitems);
    size_t r = 0, off = 0;
    for (auto &s : sl) {
        for (uint64_t len : s.lens) {
            row_ptr[r + 1] = row_ptr[r] + len;
            ++r;
        }
        std::copy(s.items.begin(), s.items.end(), items.begin() + off);
        off += s.items.size();
    }
    return SGFIM_OK;
}

static void write_env(std::ofstream &f, const sgfim_handle *h, const char *rule) {
    cudaDeviceProp prop;
    f << rule << "\n";
    if (cudaGetDeviceProperties(&prop, h->device) == cudaSuccess) {
        f << "GPU " << h->device << ": " << prop.name << "\n";
        f << "     Multi-Processor Count: " << prop.multiProcessorCount << "\n";
        f << "     Max Threads Per Multi-Processor: " << prop.maxThreadsPerMultiProcessor << "\n";
        f << "     Warp Size: " << prop.warpSize << "\n";
        f << "     Max Threads Per Block: " << prop.maxThreadsPerBlock << "\n";
        f << "     Compute Capability: " << prop.major << "." << prop.minor << "\n\n";
    }
    f << "CPU: host\n";
    f << "     Number of Logical Cores: " << std::thread::hardware_concurrency() << "\n\n";
    int rt = 0;
    cudaRuntimeGetVersion(&rt);
    f << "CUDA Version: " << rt / 1000 << "." << (rt % 1000) / 10 << "\n";
    f << rule << "\n";
}

static void write_dataset(std::ofstream &f, const sgfim_handle *h, const char *file) {
    const Dataset &ds = h->ds;
    f << "transSetFile: " << (file ? file : ds.source.c_str()) << "\n";
    f << "dimension: " << ds.n_present << "\n";
    f << "transNum: " << ds.n_txn << "\n";
    f << "itemIDmin: " << ds.id_min << "\n";
    f << "itemIDmax: " << ds.id_max << "\n";
    f << "transLengthMin: " << ds.len_min << "\n";
    f << "transLengthMax: " << ds.len_max << "\n";
    f << "transLengthMean: " << fmt_double(ds.len_mean) << "\n";
}

static void write_records(std::ofstream &f, const sgfim_result *r, uint64_t n_txn) {
    for (uint64_t i = 0; i < r->n_sets; ++i) {
        const uint64_t a = r->set_ptr[i], b = r->set_ptr[i + 1];
        f << (i + 1) << "th: " << (b - a) << " { ";
        // the reference lists items in the order they joined the set (descending ids)
        for (uint64_t k = b; k-- > a;) f << r->items[k] << " ";
        f << "}   support: " << fmt_double(n_txn ? (double)r->support[i] / (double)n_txn : 0.0)
          << "  frequency: " << r->support[i] << "\n";
    }
}

int write_tensorfim_file(const char *path, const sgfim_handle *h, const sgfim_result *r, const sgfim_tf_meta *m) {
    std::ofstream f(path);
    if (!f) return SGFIM_EIO;
    const char *rule = "==================================================================";
    write_env(f, h, rule);
    write_dataset(f, h, m ? m->trans_set_file : nullptr);
    f << "\nsupportThreshold: " << fmt_double(m ? m->support_threshold : 0.0) << "\n\n";
    f << "dimensionReduced: " << (m ? m->dimension_reduced : 0) << "\n";
    f << "transNumReduced: " << h->ds.n_txn << "\n";
    f << "\nGPUtaskPercentage: 100%\n";
    f << rule << "\n";
    const double pre = m ? m->preprocessing_time_s : 0.0, comp = m ? m->computation_time_s : r->elapsed_s;
    f << "preprocessing_time(s): " << fmt_double(pre) << "\n";
    f << "computation_time(s): " << fmt_double(comp) << "\n";
    f << "total_time(s): " << fmt_double(pre + comp) << "\n";
    f << "\nMFIsNumber: " << r->n_sets << "\n";
    f << "============================List of MFIs:=============================\n";
    write_records(f, r, h->ds.n_txn);
    f << rule << "\n";
    return f.good() ? SGFIM_OK : SGFIM_EIO;
}

int write_anyfim_file(const char *path, const sgfim_handle *h, sgfim_result *const *stages, const sgfim_af_meta *m) {
    std::ofstream f(path);
    if (!f) return SGFIM_EIO;
    const char *rule = "=================================================================";
    write_env(f, h, rule);
    write_dataset(f, h, m->trans_set_file);
    const uint32_t K = m->upto_stage;
    const double n = (double)h->ds.n_txn;
    f << "\nUptoStage: " << K << "\n";
    f << "preprocessing_time(s): " << fmt_double(m->preprocessing_time_s) << "\n";
    f << "GPUtaskPercentage: 100%\n";
    f << rule << "\n";
    f << "runtimePerStage(s):";
    for (uint32_t k = 0; k < K; ++k) f << " " << fmt_double(m->runtime_per_stage_s ? m->runtime_per_stage_s[k] : 0.0) << ",";
    f << "\n\nfrequencyThrePerStage:";
    for (uint32_t k = 0; k < K; ++k) f << " " << m->frequency_thr_per_stage[k] << ",";
    f << "\nsupportThrePerStage:";
    for (uint32_t k = 0; k < K; ++k) f << " " << fmt_double(n ? m->frequency_thr_per_stage[k] / n : 0.0) << ",";
    f << "\n\ndimensionPerStage:";
    for (uint32_t k = 0; k < K; ++k) f << " " << (k + 1) << ",";
    std::vector<uint64_t> cnt(K), its(K);
    for (uint32_t k = 0; k < K; ++k) {
        cnt[k] = stages[k] ? stages[k]->n_sets : 0;
        its[k] = stages[k] ? stages[k]->set_ptr[stages[k]->n_sets] : 0;
    }
    f << "\n\nMFIsNumPerStage:";
    for (uint32_t k = 0; k < K; ++k) f << " " << cnt[k] << ",";
    f << "\nitemsNumPerStage:";
    for (uint32_t k = 0; k < K; ++k) f << " " << its[k] << ",";
    f << "\n\nMFIsNumPerStage_withRemoveDuplicate:";
    for (uint32_t k = 0; k < K; ++k) f << " " << cnt[k] << ",";
    f << "\nitemsNumPerStage_withRemoveDuplicate:";
    for (uint32_t k = 0; k < K; ++k) f << " " << its[k] << ",";
    f << "\n";
    for (uint32_t k = 0; k < K; ++k) {
        f << "====================== " << (k + 1) << "th stage MFIs Number: " << cnt[k] << " ======================\n";
        if (stages[k]) write_records(f, stages[k], h->ds.n_txn);
        f << "\nfrequencyThreshold: " << m->frequency_thr_per_stage[k] << "\n";
    }
    f << rule << "\n";
    return f.good() ? SGFIM_OK : SGFIM_EIO;
}

}  // namespace sg
