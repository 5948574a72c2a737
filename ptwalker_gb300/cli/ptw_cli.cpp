// Command-line apps over the C ABI, with the reference apps' flag surface
// (include/option.hpp:132-302 and :304-355):
//
//   pagerank  -f text|binary -g PATH (-w W | -e E) --sp P [-l L] [--ws N] [--db D]
//   ppr       same, plus --source NAME (the reference hard-codes internal id 0,
//             src/core/ppr.cpp:54; here the source is a vertex name)
//   rwr       -f -g (-w | -e) [--sp P] (the reference fixes 0.5, RWR.cpp:122)
//   deepwalk  -f -g (-w | -e) -l L
//   node2vec  -f -g (-w | -e) -l L -p P -q Q  (src/core/node2vec.cpp,
//             include/option.hpp:447-469)
//
// -t, -s, --mem, --socket-mapping, --ws and --db size CPU thread pools and
// NUMA partitions in the reference; they are accepted and ignored.  Added:
// --seed S, --start per_vertex|uniform, --out FILE (counts by name as u32, or
// (start,end) pairs for rwr), --paths-out FILE (int32 [W, L] for deepwalk and node2vec),
// --as-undirected, --tune auto|block,ilp,chunk,hot_k[,min_blocks[,paths_ilp[,cache_hints
// [,paths_named[,ext_columns[,gather_slots[,warp_agg]]]]]]] (launch parameters; auto runs
// ptw_autotune), and for ppr --sources FILE|a,b,c (many sources in one batched launch, -w
// walkers each, or --budget learned --model FILE: per-source budgets from a budget model
// written by ptwalker_gb300.learned.BudgetModel.save; --out then holds u64 nq, u64
// offsets[nq+1], u32 names[], u32 counts[], and --budgets-out FILE the u64 budgets).  The app is chosen by the executable name or by the
// first argument (ptw_cli pagerank ...).  Like the reference apps, each
// prints "ppr value %u" (here: the count of vertex name 0) on stdout.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ptw.h"

namespace {

struct Opts {
    std::string app, fmt, path, out, paths_out, start = "per_vertex";
    std::string sources, budget = "fixed", model, tune, budgets_out;
    uint64_t walkers = 0, epochs = 0, seed = 0;
    double sp = -1, p = -1, q = -1;
    long len = -1;
    long long source = -1;
    bool undirected = false;
};

const char *kUsage =
    "usage: {pagerank|ppr|rwr|deepwalk|node2vec} -f text|binary -g PATH (-w W | -e E) [--sp P] [-l L]\n"
    "       [-p P -q Q (node2vec)] [--tune auto|block,ilp,chunk,hot_k,...]\n"
    "       [--source NAME | --sources FILE|a,b,c [--budget fixed|learned --model FILE]\n"
    "        [--budgets-out FILE]] [--seed S] [--start per_vertex|uniform] [--out FILE]\n"
    "       [--paths-out FILE] [--as-undirected] [-t T -s S --mem G --socket-mapping M\n"
    "       --ws N --db D (accepted, ignored)]\n"
    "The app is the program name (pagerank, ppr or PPR, rwr or RWR, deepwalk, node2vec) or the first\n"
    "argument.\n";

int usage(const char *msg)
{
    std::fprintf(stderr, "error: %s\n%s", msg, kUsage);
    return 1;
}

// The reference's program names (src/core/*.cpp) in lower case.
std::string app_name(std::string a)
{
    for (char &c : a) c = (char)std::tolower((unsigned char)c);
    return a;
}

const char *base_name(const char *p)
{
    const char *s = std::strrchr(p, '/');
    return s ? s + 1 : p;
}

int check(int rc, const char *what)
{
    if (rc != PTW_OK) std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, ptw_last_error());
    return rc;
}

bool write_file(const std::string &path, const void *data, size_t bytes)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}

// Source names from a file (whitespace-separated) or a comma-separated list.
bool read_sources(const std::string &arg, std::vector<uint32_t> &out)
{
    std::string text;
    if (FILE *f = std::fopen(arg.c_str(), "rb")) {
        char buf[1 << 16];
        size_t k;
        while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
        std::fclose(f);
    } else {
        text = arg;
    }
    for (char &c : text)
        if (c == ',') c = ' ';
    const char *p = text.c_str();
    char *end = nullptr;
    for (;;) {
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) break;
        const unsigned long long v = std::strtoull(p, &end, 10);
        if (end == p || v > 0xFFFFFFFFull) return false;
        out.push_back((uint32_t)v);
        p = end;
    }
    return !out.empty();
}

// Launch parameters: "auto" (ptw_autotune), or block,ilp,chunk,hot_k[,min_blocks[,paths_ilp
// [,cache_hints[,paths_named[,ext_columns[,gather_slots[,warp_agg]]]]]]] over the graph's
// current tune.
int apply_tune(ptw_graph *g, const std::string &spec, double sp, uint64_t walkers)
{
    ptw_tune t;
    if (spec == "auto") {
        if (check(ptw_autotune(g, sp > 0 ? sp : 0.15, walkers, &t), "autotune")) return 1;
        return check(ptw_graph_set_tune(g, &t), "set tune") ? 1 : 0;
    }
    if (check(ptw_graph_get_tune(g, &t), "get tune")) return 1;
    int32_t *fields[] = {&t.block, &t.ilp, &t.chunk, &t.hot_k, &t.min_blocks, &t.paths_ilp,
                         &t.cache_hints, &t.paths_named, &t.ext_columns, &t.gather_slots, &t.warp_agg};
    size_t i = 0, pos = 0;
    while (pos <= spec.size() && i < sizeof fields / sizeof fields[0]) {
        const size_t c = spec.find(',', pos);
        const std::string v = spec.substr(pos, c == std::string::npos ? std::string::npos : c - pos);
        char *end = nullptr;
        const long x = std::strtol(v.c_str(), &end, 10);
        if (v.empty() || *end) {
            std::fprintf(stderr, "error: bad --tune value %s\n", spec.c_str());
            return 1;
        }
        *fields[i++] = (int32_t)x;
        if (c == std::string::npos) break;
        pos = c + 1;
    }
    return check(ptw_graph_set_tune(g, &t), "set tune") ? 1 : 0;
}

// Per-source budgets from a budget model file (ptwalker_gb300.learned.BudgetModel.save):
// b = kappa * exp(MLP(features)), clamped to [b_min, b_max], the fallback when not finite.
int learned_budgets(ptw_graph *g, const std::string &path, const std::vector<uint32_t> &src,
                    std::vector<uint64_t> &budgets)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::fprintf(stderr, "error: cannot open model %s\n", path.c_str());
        return 1;
    }
    char magic[8];
    double kappa = 0;
    uint64_t lim[3];
    std::vector<float> params(PTW_MLP_NPARAMS), norm(PTW_MLP_NNORM);
    const bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "PTWBUD1", 8) == 0 &&
                    std::fread(&kappa, sizeof kappa, 1, f) == 1 && std::fread(lim, sizeof lim[0], 3, f) == 3 &&
                    std::fread(params.data(), 4, params.size(), f) == params.size() &&
                    std::fread(norm.data(), 4, norm.size(), f) == norm.size();
    std::fclose(f);
    if (!ok) {
        std::fprintf(stderr, "error: %s is not a budget model\n", path.c_str());
        return 1;
    }
    std::vector<float> feat(src.size() * PTW_MLP_IN), pred(src.size());
    if (check(ptw_source_features(g, src.data(), (uint32_t)src.size(), feat.data()), "source features")) return 1;
    ptw_mlp *m = nullptr;
    if (check(ptw_mlp_create(0, &m), "model")) return 1;
    int rc = check(ptw_mlp_set_params(m, params.data(), norm.data()), "model parameters");
    if (!rc) rc = check(ptw_mlp_forward(m, feat.data(), (uint32_t)src.size(), pred.data()), "model forward");
    ptw_mlp_free(m);
    if (rc) return 1;
    budgets.resize(src.size());
    for (size_t i = 0; i < src.size(); ++i) {
        double b = kappa * std::exp((double)pred[i]);
        if (!std::isfinite(b)) b = (double)lim[2];
        else b = std::min(std::max(b, (double)lim[0]), (double)lim[1]);
        budgets[i] = (uint64_t)b;
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    Opts o;
    int i = 1;
    o.app = app_name(base_name(argv[0]));
    if (o.app != "pagerank" && o.app != "ppr" && o.app != "rwr" && o.app != "deepwalk" && o.app != "node2vec") {
        if (argc < 2) return usage("missing app name");
        o.app = app_name(argv[1]);
        i = 2;
        if (o.app == "-h" || o.app == "--help") {
            std::fputs(kUsage, stdout);
            return 0;
        }
    }
    for (; i < argc; ++i) {
        std::string a = argv[i];
        std::string v;
        const size_t eq = a.find('=');
        if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
            v = a.substr(eq + 1);
            a = a.substr(0, eq);
        } else if (a != "--as-undirected" && a != "-h" && a != "--help") {
            if (i + 1 >= argc) return usage(("flag " + a + " needs a value").c_str());
            v = argv[++i];
        }
        if (a == "-f") o.fmt = v;
        else if (a == "-g") o.path = v;
        else if (a == "-w") o.walkers = std::strtoull(v.c_str(), nullptr, 10);
        else if (a == "-e") o.epochs = std::strtoull(v.c_str(), nullptr, 10);
        else if (a == "--sp") o.sp = std::atof(v.c_str());
        else if (a == "-l") o.len = std::atol(v.c_str());
        else if (a == "-p") o.p = std::atof(v.c_str());
        else if (a == "-q") o.q = std::atof(v.c_str());
        else if (a == "--source") o.source = std::atoll(v.c_str());
        else if (a == "--sources") o.sources = v;
        else if (a == "--budget") o.budget = v;
        else if (a == "--model") o.model = v;
        else if (a == "--tune") o.tune = v;
        else if (a == "--budgets-out") o.budgets_out = v;
        else if (a == "--seed") o.seed = std::strtoull(v.c_str(), nullptr, 10);
        else if (a == "--start") o.start = v;
        else if (a == "--out") o.out = v;
        else if (a == "--paths-out") o.paths_out = v;
        else if (a == "--as-undirected") o.undirected = true;
        else if (a == "-t" || a == "-s" || a == "--mem" || a == "--socket-mapping" || a == "--ws" ||
                 a == "--db") {
            // CPU pool / NUMA sizing in the reference: not used on the GPU
        } else if (a == "-h" || a == "--help") {
            std::fputs(kUsage, stdout);
            return 0;
        } else {
            return usage(("unknown flag " + a).c_str());
        }
    }
    if (o.fmt != "text" && o.fmt != "binary") return usage("-f must be text or binary");
    if (o.path.empty()) return usage("-g is required");
    if ((o.walkers == 0) == (o.epochs == 0)) return usage("give exactly one of -w and -e");
    if (o.app == "rwr" && o.sp < 0) o.sp = 0.5;
    if ((o.app == "pagerank" || o.app == "ppr") && o.sp <= 0) return usage("--sp is required");
    if ((o.app == "deepwalk" || o.app == "node2vec") && o.len < 1) return usage("-l is required for deepwalk and node2vec");
    if (o.app == "node2vec" && (o.p <= 0 || o.q <= 0)) return usage("-p and -q are required for node2vec");
    if (o.app == "ppr" && o.source < 0 && o.sources.empty()) return usage("--source or --sources is required for ppr");
    if (!o.sources.empty() && o.app != "ppr") return usage("--sources is for ppr");
    if (o.budget != "fixed" && o.budget != "learned") return usage("--budget must be fixed or learned");
    if (o.budget == "learned" && (o.model.empty() || o.sources.empty()))
        return usage("--budget learned needs --sources and --model");
    std::vector<uint32_t> srcs;
    if (!o.sources.empty() && !read_sources(o.sources, srcs)) return usage("--sources: no valid vertex names");
    if (o.start != "per_vertex" && o.start != "uniform") return usage("--start must be per_vertex or uniform");

    ptw_graph *g = nullptr;
    if (check(ptw_graph_load(o.path.c_str(), o.fmt == "text" ? PTW_FMT_TEXT : PTW_FMT_BINARY,
                             o.undirected ? 1 : 0, &g), "graph load"))
        return 2;
    ptw_graph_info info;
    ptw_graph_get_info(g, &info);
    ptw_walk_cfg cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.n_walkers = o.walkers ? o.walkers : o.epochs * (uint64_t)info.n_vertices;
    if (!o.tune.empty() && apply_tune(g, o.tune, o.sp, cfg.n_walkers)) {
        ptw_graph_free(g);
        return 3;
    }
    if (!srcs.empty()) {
        // many sources: one batched launch, query i = source i
        std::vector<uint64_t> budgets(srcs.size(), cfg.n_walkers);
        if (o.budget == "learned" && learned_budgets(g, o.model, srcs, budgets)) {
            ptw_graph_free(g);
            return 3;
        }
        std::vector<ptw_query> q(srcs.size());
        for (size_t i = 0; i < srcs.size(); ++i) {
            q[i].source = srcs[i];
            q[i].query_id = (uint32_t)i;
            q[i].budget = budgets[i];
        }
        ptw_batch_cfg bc;
        std::memset(&bc, 0, sizeof(bc));
        bc.sp = o.sp;
        bc.seed = o.seed;
        bc.app = PTW_APP_VISITS;
        ptw_batch *b = nullptr;
        int rc = check(ptw_ppr_batch(g, q.data(), (uint32_t)q.size(), &bc, &b), "ppr batch");
        uint64_t entries = 0;
        ptw_walk_stats bst;
        std::memset(&bst, 0, sizeof(bst));
        if (!rc) rc = check(ptw_batch_info(b, nullptr, &entries, &bst), "batch info");
        if (!rc && !o.out.empty()) {
            std::vector<uint64_t> off(q.size() + 1);
            std::vector<uint32_t> names(entries), counts(entries);
            rc = check(ptw_batch_export(b, off.data(), names.data(), counts.data()), "batch export");
            const uint64_t nq = q.size();
            FILE *f = rc ? nullptr : std::fopen(o.out.c_str(), "wb");
            if (!rc) {
                bool ok = f && std::fwrite(&nq, 8, 1, f) == 1 && std::fwrite(off.data(), 8, off.size(), f) == off.size() &&
                          std::fwrite(names.data(), 4, entries, f) == entries &&
                          std::fwrite(counts.data(), 4, entries, f) == entries;
                if (f) ok = std::fclose(f) == 0 && ok;
                if (!ok) rc = PTW_EIO;
            }
        }
        if (!rc && !o.budgets_out.empty() && !write_file(o.budgets_out, budgets.data(), budgets.size() * 8))
            rc = PTW_EIO;
        if (b) ptw_batch_free(b);
        if (rc == PTW_EIO) std::fprintf(stderr, "cannot write output file\n");
        if (!rc) {
            uint64_t total = 0;
            for (uint64_t x : budgets) total += x;
            std::printf("ppr queries %zu entries %llu\n", srcs.size(), (unsigned long long)entries);
            std::fprintf(stderr,
                         "{\"app\": \"ppr\", \"queries\": %zu, \"budget\": \"%s\", \"walkers\": %llu, "
                         "\"moves\": %llu, \"entries\": %llu}\n",
                         srcs.size(), o.budget.c_str(), (unsigned long long)total, (unsigned long long)bst.moves,
                         (unsigned long long)entries);
        }
        ptw_graph_free(g);
        return rc ? 3 : 0;
    }
    cfg.sp = o.sp > 0 ? o.sp : 0.0;
    cfg.seed = o.seed;
    cfg.start_mode = o.start == "uniform" ? PTW_START_UNIFORM : PTW_START_PER_VERTEX;
    uint32_t src = 0;
    if (o.app == "ppr") {
        src = (uint32_t)o.source;
        cfg.start_mode = PTW_START_SOURCES;
        cfg.h_sources = &src;
        cfg.n_sources = 1;
    }
    ptw_walk_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = PTW_OK;
    uint32_t value0 = 0;
    if (o.app == "pagerank" || o.app == "ppr") {
        std::vector<uint32_t> counts(info.id_bound);
        rc = check(ptw_pagerank(g, &cfg, counts.data(), &st), o.app.c_str());
        if (!rc) {
            value0 = counts.empty() ? 0 : counts[0];
            if (!o.out.empty() && !write_file(o.out, counts.data(), counts.size() * 4)) rc = PTW_EIO;
        }
    } else if (o.app == "rwr") {
        std::vector<uint32_t> pairs(2 * cfg.n_walkers);
        rc = check(ptw_rwr(g, &cfg, pairs.data(), &st), "rwr");
        if (!rc) {
            value0 = pairs.empty() ? 0 : pairs[1];
            if (!o.out.empty() && !write_file(o.out, pairs.data(), pairs.size() * 4)) rc = PTW_EIO;
        }
    } else if (o.app == "node2vec") {
        std::vector<int32_t> paths(cfg.n_walkers * (uint64_t)o.len);
        ptw_node2vec_stats ns;
        std::memset(&ns, 0, sizeof(ns));
        rc = check(ptw_node2vec(g, &cfg, (uint32_t)o.len, o.p, o.q, paths.data(), &ns), "node2vec");
        st.walkers = ns.walkers;
        st.moves = ns.moves;
        st.kernel_ms = ns.kernel_ms;
        st.total_ms = ns.total_ms;
        if (!rc && !o.paths_out.empty() && !write_file(o.paths_out, paths.data(), paths.size() * 4))
            rc = PTW_EIO;
    } else {
        std::vector<int32_t> paths(cfg.n_walkers * (uint64_t)o.len);
        rc = check(ptw_deepwalk(g, &cfg, (uint32_t)o.len, paths.data(), &st), "deepwalk");
        if (!rc && !o.paths_out.empty() && !write_file(o.paths_out, paths.data(), paths.size() * 4))
            rc = PTW_EIO;
    }
    if (rc == PTW_EIO) std::fprintf(stderr, "cannot write output file\n");
    if (!rc) {
        std::printf("ppr value %u\n", value0);
        std::fprintf(stderr,
                     "{\"app\": \"%s\", \"vertices\": %u, \"edges\": %llu, \"walkers\": %llu, "
                     "\"moves\": %llu, \"kernel_ms\": %.3f, \"total_ms\": %.3f}\n",
                     o.app.c_str(), info.n_vertices, (unsigned long long)info.n_edges,
                     (unsigned long long)st.walkers, (unsigned long long)st.moves, st.kernel_ms,
                     st.total_ms);
    }
    ptw_graph_free(g);
    return rc ? 3 : 0;
}
