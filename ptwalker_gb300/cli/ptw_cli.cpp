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
// --as-undirected.  The app is chosen by the executable name or by the
// first argument (ptw_cli pagerank ...).  Like the reference apps, each
// prints "ppr value %u" (here: the count of vertex name 0) on stdout.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ptw.h"

namespace {

struct Opts {
    std::string app, fmt, path, out, paths_out, start = "per_vertex";
    uint64_t walkers = 0, epochs = 0, seed = 0;
    double sp = -1, p = -1, q = -1;
    long len = -1;
    long long source = -1;
    bool undirected = false;
};

const char *kUsage =
    "usage: {pagerank|ppr|rwr|deepwalk|node2vec} -f text|binary -g PATH (-w W | -e E) [--sp P] [-l L]\n"
    "       [-p P -q Q (node2vec)]\n"
    "       [--source NAME] [--seed S] [--start per_vertex|uniform] [--out FILE]\n"
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
    if (o.app == "ppr" && o.source < 0) return usage("--source is required for ppr");
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
