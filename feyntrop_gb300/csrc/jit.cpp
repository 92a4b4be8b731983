#include "jit.hpp"
#include "kernels/aot.hpp"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <vector>

extern const char* ft_sample_body_source;   // generated at build time from kernels/sample_body.cuh

namespace ft {

static const char* kArch = "--gpu-architecture=sm_103a";

unsigned table_smem_bytes(const kernel_key& k)
{
    // staged table (unless read from global memory), then the per-thread accumulators:
    // FP64 form two doubles per slot; mixed form two doubles and two floats per slot and
    // four sample counters (a double and a float each)
    const unsigned entries = 1u << k.E;
    const unsigned tab = k.table_global ? 0u : (k.prec == 0 ? 25u * entries : 17u * entries);
    const unsigned parts = k.mode == 1 ? 4u : 2u;
    const unsigned acc = (unsigned)k.block * (parts * (unsigned)k.K * (k.prec == 0 ? 16u : 24u) + (k.prec == 0 ? 0u : 48u));
    return ((tab + 15u) & ~15u) + acc;
}

// Tables of the two-float logarithm, exponential and sine / cosine of the mixed kernels
// (FP32 values written exactly as hexadecimal literals):
//   FT_LOGTAB[3i .. 3i+2] = r_i = fl(1 / (1 + (i + 1/2)/64)), -log(r_i) as hi, lo (i < 64)
//   FT_EXPTAB[2j .. 2j+1] = 2^(j/32) as hi, lo (j < 32)
//   FT_SCTAB[4j .. 4j+3]  = sin(j pi/64) as hi, lo, cos(j pi/64) as hi, lo (j < 128)
static std::string tables_source()
{
    static const std::string text = [] {
        std::ostringstream s;
        char buf[64];
        s << "__device__ const float FT_LOGTAB[192] = {";
        for (int i = 0; i < 64; i++) {
            const float r = (float)(1.0 / (1.0 + (i + 0.5) / 64.0));
            const double nl = -std::log((double)r);
            const float hi = (float)nl, lo = (float)(nl - (double)hi);
            for (float v : {r, hi, lo}) {
                std::snprintf(buf, sizeof buf, "%af,", (double)v);
                s << buf;
            }
        }
        s << "};\n__device__ const float FT_EXPTAB[64] = {";
        for (int j = 0; j < 32; j++) {
            const double t = std::exp2(j / 32.0);
            const float hi = (float)t, lo = (float)(t - (double)hi);
            for (float v : {hi, lo}) {
                std::snprintf(buf, sizeof buf, "%af,", (double)v);
                s << buf;
            }
        }
        s << "};\n__device__ const float4 FT_SCTAB[128] = {";
        const double pi = 3.14159265358979323846;
        for (int j = 0; j < 128; j++) {
            const double sn = std::sin(j * pi / 64.0), cs = std::cos(j * pi / 64.0);
            const float sh = (float)sn, sl = (float)(sn - (double)sh), ch = (float)cs, cl = (float)(cs - (double)ch);
            s << "{";
            for (float v : {sh, sl, ch, cl}) {
                std::snprintf(buf, sizeof buf, "%af,", (double)v);
                s << buf;
            }
            s << "},";
        }
        s << "};\n";
        return s.str();
    }();
    return text;
}

// Structural pattern of the conductance-form elimination of the reduced Laplacian (the
// deleted vertex is V-1): nz[i*n+j] (i < j) marks a conductance between i and j that is
// non-zero when vertex i is eliminated (an edge, or fill from an earlier elimination),
// nzg[i] a conductance to ground, nzm[i*n+j] an entry of M^-1 (M the unit upper
// triangular factor) that can be non-zero.  The kernels skip every update on a
// structural zero (a compiler cannot drop x + 0 * y in IEEE arithmetic).
static void elimination_pattern(const kernel_key& k, std::vector<int>& nz, std::vector<int>& nzg,
                                std::vector<int>& nzm)
{
    const int n = k.V - 1;
    nz.assign((size_t)n * n, 0);
    nzg.assign(n, 0);
    nzm.assign((size_t)n * n, 0);
    for (int e = 0; e < k.E; e++) {
        const int a = k.ek[e], b = k.el[e];   // a > b
        if (a == k.V - 1)
            nzg[b] = 1;
        else
            nz[b * n + a] = 1;
    }
    for (int kk = 0; kk < n; kk++)
        for (int i = kk + 1; i < n; i++) {
            if (!nz[kk * n + i]) continue;
            if (nzg[kk]) nzg[i] = 1;
            for (int j = i + 1; j < n; j++)
                if (nz[kk * n + j]) nz[i * n + j] = 1;
        }
    for (int i = n - 1; i >= 0; i--)
        for (int j = i + 1; j < n; j++) {
            int v = nz[i * n + j];
            for (int m = i + 1; m < j && !v; m++) v = nz[i * n + m] && nzm[m * n + j];
            nzm[i * n + j] = v;
        }
}

std::string kernel_source(const kernel_key& k)
{
    std::ostringstream s;
    s << "// generated: one topology of the tropical sampling kernel\n";
    s << "#define FT_E " << k.E << "\n#define FT_V " << k.V << "\n#define FT_K " << k.K << "\n";
    s << "#define FT_LOOPS " << k.loops << "\n#define FT_RANK " << k.rank << "\n";
    s << "#define FT_PREC " << k.prec << "\n#define FT_MODE " << k.mode << "\n";
    s << "#define FT_ONLY_PSI " << k.only_psi << "\n#define FT_RECORD " << k.record << "\n";
    s << "#define FT_BLOCK " << k.block << "\n#define FT_TABLE_GLOBAL " << k.table_global << "\n";
    s << "#define FT_MINB " << k.minb << "\n#define FT_VARIANT " << k.variant << "\n";
    s << "#define FT_BATCH " << k.batch << "\n#define FT_XA_DIGITS " << kExactDigits << "\n";
    s << "#define FT_Q0 " << k.q0 << "\n";
    s << "__device__ constexpr int FT_EK[" << k.E << "] = {";
    for (int e = 0; e < k.E; e++) s << (e ? "," : "") << k.ek[e];
    s << "};\n__device__ constexpr int FT_EL[" << k.E << "] = {";
    for (int e = 0; e < k.E; e++) s << (e ? "," : "") << k.el[e];
    s << "};\n";
    {
        std::vector<int> nz, nzg, nzm;
        elimination_pattern(k, nz, nzg, nzm);
        const int n = k.V - 1;
        auto matrix = [&](const char* name, const std::vector<int>& m) {
            s << "__device__ constexpr unsigned char " << name << "[" << n << "][" << n << "] = {";
            for (int i = 0; i < n; i++) {
                s << "{";
                for (int j = 0; j < n; j++) s << (j ? "," : "") << m[i * n + j];
                s << "},";
            }
            s << "};\n";
        };
        matrix("FT_NZC", nz);
        matrix("FT_NZM", nzm);
        s << "__device__ constexpr unsigned char FT_NZG[" << n << "] = {";
        for (int i = 0; i < n; i++) s << (i ? "," : "") << nzg[i];
        s << "};\n#define FT_HAVE_PATTERN 1\n";
    }
    s << tables_source();
    s << ft_sample_body_source;
    return s.str();
}

static uint64_t fnv1a(const std::string& s)
{
    uint64_t h = 1469598103934665603ULL;
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ULL;
    }
    return h;
}

std::string cache_dir()
{
    if (const char* env = std::getenv("FEYNTROP_GB300_CACHE")) return env;
    Dl_info info;
    if (dladdr((void*)&cache_dir, &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        size_t slash = p.rfind('/');
        if (slash != std::string::npos) return p.substr(0, slash) + "/../_jit_cache";
    }
    return "_jit_cache";
}

static std::vector<std::string> options()
{
    return {kArch, "--std=c++17", "-lineinfo", "--extra-device-vectorization"};
}

static std::string compile(const std::string& src, std::string* log_out)
{
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "ft_sample.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        throw std::runtime_error("nvrtcCreateProgram failed");
    std::vector<std::string> opts = options();
    std::vector<const char*> o;
    for (auto& x : opts) o.push_back(x.c_str());
    if (std::getenv("FEYNTROP_GB300_PTXAS_VERBOSE")) o.push_back("--ptxas-options=-v");
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)o.size(), o.data());
    size_t logn = 0;
    nvrtcGetProgramLogSize(prog, &logn);
    std::string log(logn, '\0');
    if (logn) nvrtcGetProgramLog(prog, &log[0]);
    if (log_out) *log_out = log;
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        throw std::runtime_error("kernel compilation failed:\n" + log);
    }
    if (std::getenv("FEYNTROP_GB300_PTXAS_VERBOSE")) std::fprintf(stderr, "%s\n", log.c_str());
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::string cubin(n, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return cubin;
}

static std::string cubin_for(const kernel_key& key, double* seconds)
{
    const std::string src = kernel_source(key);
    std::string tag = src;
    for (auto& o : options()) tag += o;
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    tag += std::to_string(major) + "." + std::to_string(minor);
    char name[64];
    std::snprintf(name, sizeof name, "%016llx.cubin", (unsigned long long)fnv1a(tag));
    const std::string dir = cache_dir();
    const std::string path = dir + "/" + name;
    {
        std::ifstream f(path, std::ios::binary);
        if (f) {
            std::stringstream b;
            b << f.rdbuf();
            std::string s = b.str();
            if (!s.empty()) {
                *seconds = 0;
                return s;
            }
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    std::string cubin = compile(src, nullptr);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    mkdir(dir.c_str(), 0755);
    const std::string tmp = path + ".tmp" + std::to_string((unsigned long long)fnv1a(std::to_string((long)&tag)));
    {
        std::ofstream f(tmp, std::ios::binary);
        f.write(cubin.data(), (std::streamsize)cubin.size());
    }
    std::rename(tmp.c_str(), path.c_str());
    return cubin;
}

size_t compile_only(const kernel_key& key, std::string* log) { return compile(kernel_source(key), log).size(); }

void precompile(const kernel_key& key)
{
    double s = 0;
    cubin_for(key, &s);
}

void precompile_all(const std::vector<kernel_key>& keys)
{
    if (keys.size() < 2) {
        for (const kernel_key& k : keys) precompile(k);
        return;
    }
    // at most 8 at a time: a compile of the larger kernels takes about a gigabyte
    const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    const size_t nthreads = std::min<size_t>(keys.size(), hw);
    std::atomic<size_t> next{0};
    std::vector<std::exception_ptr> errs(nthreads);
    std::vector<std::thread> pool;
    for (size_t t = 0; t < nthreads; t++)
        pool.emplace_back([&, t] {
            try {
                for (size_t i; (i = next++) < keys.size();) precompile(keys[i]);
            } catch (...) {
                errs[t] = std::current_exception();
            }
        });
    for (auto& th : pool) th.join();
    for (auto& e : errs)
        if (e) std::rethrow_exception(e);
}

// Driver entry points are fetched through the runtime (no link-time dependency on
// the driver library, so the library also loads on machines without a GPU).
driver_api& drv()
{
    static driver_api d;
    static std::once_flag once;
    std::call_once(once, [] {
        auto get = [](const char* name, void** fn) {
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
                q != cudaDriverEntryPointSuccess || !*fn)
                throw std::runtime_error(std::string("driver entry point unavailable: ") + name);
        };
        get("cuModuleLoadData", (void**)&d.ModuleLoadData);
        get("cuModuleGetFunction", (void**)&d.ModuleGetFunction);
        get("cuFuncSetAttribute", (void**)&d.FuncSetAttribute);
        get("cuFuncGetAttribute", (void**)&d.FuncGetAttribute);
        get("cuOccupancyMaxActiveBlocksPerMultiprocessor", (void**)&d.OccupancyMaxActiveBlocksPerMultiprocessor);
        get("cuLaunchKernel", (void**)&d.LaunchKernel);
        get("cuGetErrorString", (void**)&d.GetErrorString);
    });
    return d;
}

void check(CUresult r, const char* what)
{
    if (r != CUDA_SUCCESS) {
        const char* msg = nullptr;
        drv().GetErrorString(r, &msg);
        throw std::runtime_error(std::string(what) + ": " + (msg ? msg : "unknown driver error"));
    }
}

static std::string key_string(const kernel_key& k)
{
    std::ostringstream s;
    s << k.E << "," << k.V << "," << k.K << "," << k.loops << "," << k.rank << "," << k.prec << "," << k.mode << ","
      << k.only_psi << "," << k.record << "," << k.block << "," << k.table_global << "," << k.minb << "," << k.variant
      << "," << k.batch << "," << k.q0;
    for (int e = 0; e < k.E; e++) s << ";" << k.ek[e] << "-" << k.el[e];
    return s.str();
}

static std::mutex g_mu;
static std::map<std::pair<int, std::string>, kernel_set> g_loaded;

const kernel_set* find_kernels(const kernel_key& key)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_loaded.find(std::make_pair(dev, key_string(key)));
    return it == g_loaded.end() ? nullptr : &it->second;
}

const kernel_set& get_kernels(const kernel_key& key)
{
    auto& mu = g_mu;
    auto& loaded = g_loaded;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) throw std::runtime_error("no CUDA device");
    auto k = std::make_pair(dev, key_string(key));
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = loaded.find(k);
        if (it != loaded.end()) return it->second;
    }
    // compile (or read the disk cache) outside the lock, so that threads loading
    // different kernels compile them concurrently
    kernel_set ks;
    ks.block = key.block;
    ks.variant = key.variant;
    const std::string cubin = cubin_for(key, &ks.compile_seconds);
    std::lock_guard<std::mutex> lock(mu);
    auto it = loaded.find(k);
    if (it != loaded.end()) return it->second;   // another thread loaded it meanwhile
    cudaFree(0);   // make the runtime's primary context current for the driver calls
    check(drv().ModuleLoadData(&ks.module, cubin.data()), "cuModuleLoadData");
    const char* sname = key.batch ? "ft_sample_batch" : "ft_sample";
    const char* qname = key.batch ? "ft_sample_queue_batch" : "ft_sample_queue";
    check(drv().ModuleGetFunction(&ks.sample, ks.module, sname), "cuModuleGetFunction(sampling kernel)");
    if (key.prec == 0) check(drv().ModuleGetFunction(&ks.queue, ks.module, qname), "cuModuleGetFunction(queue)");
    ks.smem = table_smem_bytes(key);
    CUfunction fs[2] = {ks.sample, ks.queue};
    for (CUfunction f : fs) {
        if (!f) continue;
        check(drv().FuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)ks.smem),
              "cuFuncSetAttribute(smem)");
    }
    check(drv().FuncGetAttribute(&ks.regs, CU_FUNC_ATTRIBUTE_NUM_REGS, ks.sample), "cuFuncGetAttribute");
    check(drv().FuncGetAttribute(&ks.local_bytes, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, ks.sample), "cuFuncGetAttribute");
    check(drv().OccupancyMaxActiveBlocksPerMultiprocessor(&ks.blocks_per_sm, ks.sample, ks.block, ks.smem),
          "cuOccupancyMaxActiveBlocksPerMultiprocessor");
    if (ks.queue)
        check(drv().OccupancyMaxActiveBlocksPerMultiprocessor(&ks.queue_blocks_per_sm, ks.queue, ks.block, ks.smem),
              "cuOccupancyMaxActiveBlocksPerMultiprocessor");
    if (ks.blocks_per_sm < 1) throw std::runtime_error("sampling kernel does not fit on an SM");
    return loaded.emplace(k, ks).first->second;
}

}  // namespace ft
