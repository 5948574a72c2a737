// Driver around the reference's own pagerank app (TEST INFRASTRUCTURE: the
// CPU baseline and the statistical pin of the oracle; never part of the
// engine).
//
// It compiles src/core/pagerank.cpp unmodified (its main is renamed so this
// file can supply one), together with the reference headers it includes, and
// runs the same sequence as that main (src/core/pagerank.cpp:93-112) and the
// free walk() (src/core/solver.hpp:1049-1074): Graph::load, the app `PPR`,
// FMobSolver prepare / generate_walkers, then the timed epoch loop.
//
// What it adds, because the reference prints only one counter:
//  * the visit counts are written out by vertex name.  Graph::load deletes
//    its relabelling table (`delete []reorderid`, src/core/graph.hpp:672) but
//    leaves the member pointer set; array deletes are deferred while load()
//    runs so the table stays readable.  The first-appearance name compaction
//    (graph.hpp:293-311) is recomputed from the same edge file.
//  * steps = sum(visits) - W (the reference never increments its step
//    counter, solver.hpp:676,924,1070).
//
// Usage: ptw_ref_walk -f text|binary -g PATH (-w W | -e E) --sp P [-t T]
//                     [--db D] [--out COUNTS.u32] [--json RESULT.json] [--reps R]
#include <cstdlib>
#include <new>

static bool g_defer_array_delete = false;

void *operator new[](std::size_t n)
{
    void *p = std::malloc(n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void *operator new[](std::size_t n, const std::nothrow_t &) noexcept { return std::malloc(n ? n : 1); }
void operator delete[](void *p) noexcept
{
    if (!g_defer_array_delete) std::free(p);
}
void operator delete[](void *p, std::size_t) noexcept
{
    if (!g_defer_array_delete) std::free(p);
}

#define main ptw_reference_pagerank_main
#include "pagerank.cpp"
#undef main

#include <cstring>
#include <fstream>
#include <thread>

static uint64_t l2_bytes()
{
    // Per-core L2 as the reference's get_l2_cache_size() reports it
    // (include/sysinfo.hpp:62-71), with a sysfs fallback for hosts where
    // getconf has no cache data (e.g. aarch64).
    uint64_t v = get_l2_cache_size();
    if (v) return v;
    std::ifstream f("/sys/devices/system/cpu/cpu0/cache/index2/size");
    std::string s;
    if (f >> s) {
        uint64_t x = std::strtoull(s.c_str(), nullptr, 10);
        if (!s.empty() && (s.back() == 'K' || s.back() == 'k')) x <<= 10;
        if (!s.empty() && (s.back() == 'M' || s.back() == 'm')) x <<= 20;
        if (x) return x;
    }
    return 1u << 20;
}

static int usage()
{
    std::fprintf(stderr,
                 "usage: ptw_ref_walk -f text|binary -g PATH (-w W | -e E) --sp P [-t T] [--db D]\n"
                 "                    [--out COUNTS.u32] [--json RESULT.json] [--reps R]\n");
    return 2;
}

int main(int argc, char **argv)
{
    std::string fmt = "text", path, out, json;
    uint64_t walkers = 0, epochs = 0;
    double sp = -1;
    int threads = (int)std::thread::hardware_concurrency();
    vertex_id_t db = 32;
    int reps = 1;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> std::string { return i + 1 < argc ? argv[++i] : std::string(); };
        if (a == "-f") fmt = next();
        else if (a == "-g") path = next();
        else if (a == "-w") walkers = std::strtoull(next().c_str(), nullptr, 10);
        else if (a == "-e") epochs = std::strtoull(next().c_str(), nullptr, 10);
        else if (a == "--sp") sp = std::atof(next().c_str());
        else if (a == "-t") threads = std::atoi(next().c_str());
        else if (a == "--db") db = (vertex_id_t)std::strtoul(next().c_str(), nullptr, 10);
        else if (a == "--out") out = next();
        else if (a == "--json") json = next();
        else if (a == "--reps") reps = std::atoi(next().c_str());
        else return usage();
    }
    if (path.empty() || sp <= 0 || sp > 1 || (walkers == 0) == (epochs == 0) || threads < 1 || reps < 1)
        return usage();

    MultiThreadConfig mtcfg;
    mtcfg.thread_num = threads;
    mtcfg.socket_num = 1;
    mtcfg.set_default_socket_mapping();
    mtcfg.l2_cache_size = l2_bytes();
    omp_set_dynamic(0);
    omp_set_num_threads(threads);
    const GraphFormat gf = fmt == "binary" ? BinaryGraphFormat : TextGraphFormat;

    Timer load_timer;
    Graph graph(mtcfg);
    try {
        g_defer_array_delete = true;
        graph.load(path.c_str(), gf, false, db);
        g_defer_array_delete = false;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "reference Graph::load failed: %s\n", e.what());
        return 3;
    }
    const double load_s = load_timer.duration();

    // First-appearance compaction of names, as Graph::load does it.
    std::vector<Edge> edges;
    if (gf == BinaryGraphFormat) read_binary_graph(path.c_str(), edges);
    else read_text_graph(path.c_str(), edges);
    std::vector<uint32_t> name2id;
    uint32_t next_id = 0, id_bound = 0;
    for (const Edge &e : edges) {
        for (uint32_t nm : {e.src, e.dst}) {
            if (nm >= name2id.size()) name2id.resize((size_t)nm + 1, UINT32_MAX);
            if (name2id[nm] == UINT32_MAX) name2id[nm] = next_id++;
            id_bound = std::max(id_bound, nm + 1);
        }
    }
    std::vector<Edge>().swap(edges);
    if (next_id != graph.v_num_old) {
        std::fprintf(stderr, "vertex count mismatch: %u vs %u\n", next_id, graph.v_num_old);
        return 4;
    }

    const uint64_t W = walkers ? walkers : epochs * (uint64_t)graph.v_num_old;
    const int walk_len = int(1 / sp) + 1;  // RWPTWalkOptionHelper default, option.hpp:270
    std::vector<double> secs;
    std::vector<uint32_t> counts(id_bound, 0);
    uint64_t visits = 0;
    for (int r = 0; r < reps; ++r) {
        PPR myapp(sp, &graph);
        FMobSolver solver(&graph, mtcfg);
        solver.prepare(W, walk_len, get_sys_mem(), 4196);
        solver.generate_walkers();
        Timer tottimer;  // the reference's timed region, solver.hpp:1055-1073
        while (solver.has_next_walk()) {
            walker_id_t epoch_walker_num = solver.get_epoch_walker_num();
            solver.walk(epoch_walker_num, myapp);
        }
        secs.push_back(tottimer.duration());
        if (r == reps - 1) {
            visits = 0;
            for (vertex_id_t v = 0; v < graph.v_num; ++v) visits += myapp.rooted_value[v];
            for (uint32_t nm = 0; nm < name2id.size(); ++nm)
                if (name2id[nm] != UINT32_MAX) counts[nm] = myapp.rooted_value[graph.reorderid[name2id[nm]]];
        }
    }
    if (!out.empty()) {
        FILE *f = std::fopen(out.c_str(), "wb");
        if (!f || std::fwrite(counts.data(), 4, counts.size(), f) != counts.size()) return 5;
        std::fclose(f);
    }
    std::ostringstream js;
    js << "{\"walkers\": " << W << ", \"visits\": " << visits << ", \"steps\": " << (visits - W)
       << ", \"threads\": " << threads << ", \"vertices\": " << graph.v_num_old
       << ", \"edges\": " << graph.e_num << ", \"id_bound\": " << id_bound << ", \"load_s\": " << load_s
       << ", \"walk_s\": [";
    for (size_t i = 0; i < secs.size(); ++i) js << (i ? ", " : "") << secs[i];
    js << "]}";
    if (!json.empty()) {
        std::ofstream jf(json);
        jf << js.str() << "\n";
    }
    std::fprintf(stderr, "%s\n", js.str().c_str());
    return 0;
}
