#include "tune.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

#include "json.hpp"

namespace ft {

namespace {

std::mutex g_mu;
std::map<std::string, launch_shape> g_table;
bool g_loaded = false;

const unsigned kSmemLimit = 227 * 1024;

std::string table_path() { return cache_dir() + "/tuning.json"; }

void load_locked()
{
    if (g_loaded) return;
    g_loaded = true;
    std::ifstream f(table_path());
    if (!f) return;
    std::stringstream b;
    b << f.rdbuf();
    try {
        const ftj::value v = ftj::parse(b.str());
        if (!v.is_object()) return;
        for (const auto& kv : v.obj) {
            const ftj::value& e = kv.second;
            if (!e.is_object()) continue;
            launch_shape s;
            s.block = (int)e["block"].num;
            s.minb = (int)e["minb"].num;
            s.variant = (int)e["variant"].num;
            s.chunk = (unsigned long long)e["chunk"].num;
            s.rate = e["rate"].num;
            if (s.block >= 32 && s.block <= 1024 && s.minb >= 1 && s.minb <= 32) g_table[kv.first] = s;
        }
    } catch (...) {
        // an unreadable table is ignored (defaults apply)
    }
}

void save_locked()
{
    std::ostringstream o;
    o << "{\n";
    bool first = true;
    for (const auto& kv : g_table) {
        const launch_shape& s = kv.second;
        o << (first ? "" : ",\n") << "  \"" << kv.first << "\": {\"block\": " << s.block << ", \"minb\": " << s.minb
          << ", \"variant\": " << s.variant << ", \"chunk\": " << s.chunk << ", \"rate\": " << s.rate << "}";
        first = false;
    }
    o << "\n}\n";
    const std::string path = table_path();
    const std::string tmp = path + ".tmp";
    {
        std::ofstream f(tmp);
        f << o.str();
    }
    std::rename(tmp.c_str(), path.c_str());
}

}  // namespace

std::string tune_class(const kernel_key& k)
{
    std::ostringstream s;
    s << "E" << k.E << "V" << k.V << "K" << k.K << "m" << k.mode << "p" << k.prec << "t" << k.table_global << "o"
      << k.only_psi << ":";
    for (size_t e = 0; e < k.ek.size(); e++) s << (e ? "," : "") << k.ek[e] << "-" << k.el[e];
    return s.str();
}

launch_shape default_shape(const kernel_key& k)
{
    // GB300 sweeps (double box, box-pentagon, 3-loop ladder, K4, cube): the mixed form is
    // bound by instruction fetch and gains 15-25 % from blocks whose warps start each
    // sample together (variant bit 2).  Deformed integrands, whose determinant and V run
    // in two-float, gain most from a smaller code: one out-of-line copy of the FP32
    // transcendentals (bit 0), of the larger two-float routines (bit 3) and of the
    // complex two-float product and multiply-add (bit 4: +37 % on the double box, +82 %
    // on the box-pentagon).  With it they run best as two 256-thread blocks per SM
    // (128 registers; double box 1.59e9 samples/s, 3-loop ladder 7.2e8; the box-pentagon
    // 0.94e9 against 1.01e9 for 512 x 1).  Out-of-line two-float add and multiply (bit 1)
    // cost 45 %.  Undeformed integrands keep one 512-thread block.  The FP64 form is
    // FP64-pipe bound (256 x 1); the per-sample barrier keeps its warps from drifting
    // apart too (cube +10 %, double box +1 %).
    launch_shape s;
    if (k.prec == 1) {
        s.block = k.mode == 1 ? 256 : 512;
        s.minb = k.mode == 1 ? 2 : 1;
    } else {
        s.block = 256;
        s.minb = 1;
    }
    s.variant = (k.prec == 1 && k.mode == 1) ? 29 : (k.mode == 1 ? 5 : 4);
    return s;
}

// Shared memory of one block: the dynamic part (staged table, per-thread sums) plus the
// kernel body's static arrays, the block reduction's per-warp slots and, in the batch
// kernels, the staged parameter block (its doubles, floats and two-float pairs) and the
// work-item variables.
static unsigned block_smem_bytes(const kernel_key& k)
{
    const unsigned slots = 8u * (unsigned)k.K + 8u;
    const unsigned red = (unsigned)(k.block / 32) * slots * 8u;
    unsigned prm = 0;
    if (k.batch) {
        const unsigned n = (unsigned)(k.V - 1), ne = n - (unsigned)k.q0, r = (unsigned)k.rank;
        const unsigned p = 8u + 2u * (unsigned)k.E + r + r * n + ne * (ne + 1u) / 2u;
        prm = (p + (p + 1u) / 2u + p) * 8u + 64u;
    }
    return table_smem_bytes(k) + red + prm;
}

void apply_shape(kernel_key& k, const launch_shape& s)
{
    k.block = s.block;
    k.minb = s.minb;
    k.variant = s.variant;
    // keep the warps per SM while halving the block until the shared memory fits
    while (k.block > 64 && block_smem_bytes(k) > kSmemLimit) {
        k.block /= 2;
        k.minb = k.minb * 2 > 32 ? 32 : k.minb * 2;
    }
}

launch_shape choose_shape(const kernel_key& k)
{
    launch_shape s = default_shape(k);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        load_locked();
        auto it = g_table.find(tune_class(k));
        if (it != g_table.end()) s = it->second;
    }
    if (const char* e = std::getenv("FEYNTROP_GB300_BLOCK")) s.block = std::atoi(e);
    if (const char* e = std::getenv("FEYNTROP_GB300_MINB")) s.minb = std::atoi(e);
    if (const char* e = std::getenv("FEYNTROP_GB300_VARIANT")) s.variant = std::atoi(e);
    return s;
}

void record_shape(const kernel_key& k, const launch_shape& s)
{
    std::lock_guard<std::mutex> lock(g_mu);
    load_locked();
    g_table[tune_class(k)] = s;
    save_locked();
}

static thread_local unsigned long long t_chunk_override = 0;
void set_chunk_override(unsigned long long chunk) { t_chunk_override = chunk; }
unsigned long long chunk_override() { return t_chunk_override; }

void clear_shapes()
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_table.clear();
    g_loaded = true;
}

}  // namespace ft
