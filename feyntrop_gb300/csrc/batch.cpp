// Batches: many integrals, of one or several topologies, in one CUDA graph launch.
//
// A batch groups its plans by kernel class (topology, eps orders, regime, table
// placement): each class is one persistent launch of ft_sample_batch, whose blocks
// take work items (FT_BLOCK * chunk consecutive samples of one integral) from a device
// counter until all items of all the class's integrals are done.  The classes run
// side by side on forked streams.  One run is
//   1. one host-to-device copy of the per-run descriptors (N, seed state, first item of
//      every integral, and each class's item total with its counters zeroed),
//   2. per class: the item stream states (one warp per integral, GF(2) skip-ahead),
//      the persistent sampling launch, in mixed precision the FP64 pass over the
//      handed-off samples, and the per-integral reduction,
//   3. one device-to-host copy of every integral's sums and the classes' counters,
// captured once into a CUDA graph and replayed while the batch's capacities hold.
// Results are those of ft_integrate on the same samples (the same sample stream per
// integral), up to the order of the floating-point sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "kernels/aot.hpp"
#include "plan.hpp"

using namespace ftrt;

namespace {

// device descriptor layouts (sample_body.cuh: batch_inst; aot.cu: item_prep)
struct batch_inst {
    const double* prm;
    const unsigned char* tab;
    unsigned long long nsamples, first_item, nitems, pad[3];
};
struct item_prep {
    unsigned long long s[4];
    unsigned long long skip;
    unsigned long long first_item, nitems, pad;
};
static_assert(sizeof(batch_inst) == 64 && sizeof(item_prep) == 64, "descriptor layout");

// per-class counters, copied in (zeroed) and out every run
struct class_header {
    unsigned long long total_items;
    unsigned long long counter;   // next work item
    unsigned long long qcount;    // FP64 hand-offs (the kernel counts in the low 32 bits)
    unsigned long long pad;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

struct ft_batch {
    struct group {
        ft::kernel_key key;                     // the class's batch sampling module
        const ft::kernel_set* ks = nullptr;
        const ft::kernel_set* k64 = nullptr;    // FP64 batch module (queue kernel), mixed only
        std::vector<int> members;               // indices into plans
        int K = 1, rank = 1, draws = 1;
        unsigned long long chunk = 64;
        int lanebits = 8;
        unsigned grid = 0, qgrid = 0;
        size_t prm_stride = 0, tab_stride = 0;  // bytes
        // offsets of this class's records in the run descriptors
        size_t off_hdr = 0, off_inst = 0, off_prep = 0, off_out = 0, off_qacc = 0;
        unsigned char* d_prm = nullptr;
        unsigned char* d_tab = nullptr;
        unsigned long long* d_lanepw = nullptr;
        unsigned long long* d_itemM = nullptr;
        unsigned long long* d_item_state = nullptr;
        size_t item_cap = 0;
        double* d_parts = nullptr;
        unsigned long long* d_queue = nullptr;
        size_t qcap = 0;
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        unsigned long long total_items = 0;
    };

    std::vector<ft_plan*> plans;
    int precision = 0;
    int device = 0;
    std::vector<group> groups;
    std::vector<int> group_of, slot_of;     // per plan: class and position in it
    // run descriptors: [class headers][batch_inst records][item_prep records], copied in
    size_t desc_bytes = 0, hdr_bytes = 0, out_doubles = 0, qacc_words = 0;
    unsigned char* h_desc = nullptr;
    unsigned char* d_desc = nullptr;
    double* d_out = nullptr;     // per integral 8K+8 sums
    double* h_out = nullptr;
    class_header* h_hdr_out = nullptr;
    unsigned long long* d_qacc = nullptr;   // per integral the FP64 pass's exact accumulators (exact_words)
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t exec = nullptr;
    int captures = 0;
    int launches = 0;
    double last_ms = 0;
    std::mutex mu;

    ~ft_batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        for (group& g : groups) {
            cudaFree(g.d_prm);
            cudaFree(g.d_tab);
            cudaFree(g.d_lanepw);
            cudaFree(g.d_itemM);
            cudaFree(g.d_item_state);
            cudaFree(g.d_parts);
            cudaFree(g.d_queue);
            if (g.stream) cudaStreamDestroy(g.stream);
            if (g.done) cudaEventDestroy(g.done);
        }
        if (h_desc) cudaFreeHost(h_desc);
        if (h_out) cudaFreeHost(h_out);
        if (h_hdr_out) cudaFreeHost(h_hdr_out);
        cudaFree(d_desc);
        cudaFree(d_out);
        cudaFree(d_qacc);
        if (stream) cudaStreamDestroy(stream);
        if (fork) cudaEventDestroy(fork);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }
};

namespace {

std::string class_id(const ft::kernel_key& k)
{
    std::string s = std::to_string(k.E) + "," + std::to_string(k.V) + "," + std::to_string(k.K) + "," +
                    std::to_string(k.loops) + "," + std::to_string(k.mode) + "," + std::to_string(k.only_psi) + "," +
                    std::to_string(k.table_global) + "," + std::to_string(k.prec);
    for (size_t e = 0; e < k.ek.size(); e++) s += ";" + std::to_string(k.ek[e]) + "-" + std::to_string(k.el[e]);
    return s;
}

// parameter block of plan pl laid out for rank R (sigma and q padded with zeros)
std::vector<double> padded_params(const ft_plan& pl, int R)
{
    const int E = pl.P.E, n = pl.P.V - 1, r0 = (int)pl.sigma.size();
    const size_t tail = pl.prm.size() - (8 + 2 * E + r0 + (size_t)r0 * n);   // P~'s external block
    std::vector<double> p(8 + 2 * E + R + (size_t)R * n + tail, 0.0);
    std::copy(pl.prm.begin(), pl.prm.begin() + 8 + 2 * E, p.begin());
    for (int r = 0; r < r0; r++) {
        p[8 + 2 * E + r] = pl.sigma[r];
        for (int i = 0; i < n; i++) p[8 + 2 * E + R + (size_t)r * n + i] = pl.q[(size_t)r * n + i];
    }
    std::copy(pl.prm.end() - tail, pl.prm.end(), p.end() - tail);
    return p;
}

unsigned long long env_u64(const char* name, unsigned long long dflt)
{
    const char* e = std::getenv(name);
    return e ? std::strtoull(e, nullptr, 10) : dflt;
}

void build(ft_batch& b)
{
    const int prec = b.precision;
    std::map<std::string, int> ids;
    b.group_of.assign(b.plans.size(), -1);
    b.slot_of.assign(b.plans.size(), -1);
    for (size_t i = 0; i < b.plans.size(); i++) {
        ft_plan* pl = b.plans[i];
        if (!pl) throw std::invalid_argument("ft_batch_create: NULL plan");
        if (pl->device != b.device) throw std::invalid_argument("ft_batch_create: plans on different devices");
        const ft::kernel_key k = pl->key(prec, 0);
        const std::string id = class_id(k);
        auto it = ids.find(id);
        if (it == ids.end()) {
            it = ids.emplace(id, (int)b.groups.size()).first;
            b.groups.emplace_back();
            b.groups.back().key = k;
        }
        ft_batch::group& g = b.groups[it->second];
        b.group_of[i] = it->second;
        b.slot_of[i] = (int)g.members.size();
        g.members.push_back((int)i);
        g.rank = std::max(g.rank, (int)pl->sigma.size());
    }
    const device_state& ds = dev_state();
    // every class's kernels (and, mixed, the FP64 ones its hand-offs run on), compiled
    // concurrently before they are loaded one by one
    std::vector<ft::kernel_key> keys, keys64;
    for (ft_batch::group& g : b.groups) {
        g.key.rank = g.rank;
        g.key.batch = 1;
        keys.push_back(g.key);
        ft::kernel_key k64 = b.plans[g.members[0]]->key(0, 0);
        k64.rank = g.rank;
        k64.batch = 1;
        keys64.push_back(k64);
    }
    {
        std::vector<ft::kernel_key> all = keys;
        if (prec) all.insert(all.end(), keys64.begin(), keys64.end());
        ft::precompile_all(all);
    }
    size_t hdr = 0, inst = 0, prep = 0;
    for (size_t gi = 0; gi < b.groups.size(); gi++) {
        ft_batch::group& g = b.groups[gi];
        const ft_plan& p0 = *b.plans[g.members[0]];
        g.K = p0.P.K;
        g.draws = 2 * p0.P.E - 1;
        g.ks = &ft::get_kernels(g.key);
        if (prec) g.k64 = &ft::get_kernels(keys64[gi]);
        const ft::launch_shape tuned = ft::choose_shape(g.key);
        g.chunk = ft::chunk_override()
                      ? ft::chunk_override()
                      : env_u64("FEYNTROP_GB300_BATCH_CHUNK", tuned.chunk ? tuned.chunk : (prec ? 128 : 16));
        if (g.chunk < 1 || g.chunk >= (1ull << 18)) throw std::invalid_argument("batch chunk out of range");
        g.lanebits = 1;
        while ((1 << g.lanebits) < g.ks->block) g.lanebits++;
        g.grid = (unsigned)(ds.sms * g.ks->blocks_per_sm);
        g.qgrid = prec ? (unsigned)(ds.sms * 2) : 0;
        // parameter blocks and tables of the class's integrals
        const size_t nm = g.members.size();
        const std::vector<double> blk0 = param_block(padded_params(p0, g.rank));
        g.prm_stride = align_up(blk0.size() * 8, 256);
        g.tab_stride = align_up(p0.tab.size(), 256);
        std::vector<unsigned char> hp(g.prm_stride * nm, 0), ht(g.tab_stride * nm, 0);
        for (size_t m = 0; m < nm; m++) {
            const ft_plan& pl = *b.plans[g.members[m]];
            const std::vector<double> blk = param_block(padded_params(pl, g.rank));
            std::memcpy(hp.data() + m * g.prm_stride, blk.data(), blk.size() * 8);
            std::memcpy(ht.data() + m * g.tab_stride, pl.tab.data(), pl.tab.size());
        }
        cu(cudaMalloc(&g.d_prm, hp.size()), "cudaMalloc(batch parameters)");
        cu(cudaMalloc(&g.d_tab, ht.size()), "cudaMalloc(batch tables)");
        cu(cudaMemcpy(g.d_prm, hp.data(), hp.size(), cudaMemcpyHostToDevice), "cudaMemcpy(batch parameters)");
        cu(cudaMemcpy(g.d_tab, ht.data(), ht.size(), cudaMemcpyHostToDevice), "cudaMemcpy(batch tables)");
        // lane skip matrices (T^(chunk draws))^(2^b) and the item step T^(block chunk draws)
        cu(cudaMalloc(&g.d_lanepw, (size_t)g.lanebits * 1024 * 8), "cudaMalloc(lane skip matrices)");
        cu(cudaMalloc(&g.d_itemM, 1024 * 8), "cudaMalloc(item skip matrix)");
        cu(ft::launch_lane_powers(ds.tpow, g.chunk * g.draws, g.lanebits, g.d_lanepw, 0), "lane skip matrices");
        cu(ft::launch_lane_powers(ds.tpow, (unsigned long long)g.ks->block * g.chunk * g.draws, 1, g.d_itemM, 0),
           "item skip matrix");
        cu(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking), "cudaStreamCreate");
        cu(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming), "cudaEventCreate");
        g.off_hdr = hdr;
        hdr += sizeof(class_header);
        g.off_inst = inst;
        inst += nm * sizeof(batch_inst);
        g.off_prep = prep;
        prep += nm * sizeof(item_prep);
        g.off_out = b.out_doubles;
        b.out_doubles += nm * (8 * g.K + 8);
        g.off_qacc = b.qacc_words;
        b.qacc_words += nm * ft::exact_words(g.K);
    }
    b.hdr_bytes = align_up(hdr, 64);
    const size_t inst_base = b.hdr_bytes, prep_base = inst_base + inst;
    for (ft_batch::group& g : b.groups) {
        g.off_inst += inst_base;
        g.off_prep += prep_base;
    }
    b.desc_bytes = prep_base + prep;
    cu(cudaMallocHost(&b.h_desc, b.desc_bytes), "cudaMallocHost(batch descriptors)");
    cu(cudaMalloc(&b.d_desc, b.desc_bytes), "cudaMalloc(batch descriptors)");
    cu(cudaMallocHost(&b.h_out, b.out_doubles * 8), "cudaMallocHost(batch results)");
    cu(cudaMallocHost(&b.h_hdr_out, b.hdr_bytes), "cudaMallocHost(batch counters)");
    cu(cudaMalloc(&b.d_out, b.out_doubles * 8), "cudaMalloc(batch results)");
    if (prec) cu(cudaMalloc(&b.d_qacc, b.qacc_words * 8), "cudaMalloc(batch FP64-pass sums)");
    std::memset(b.h_desc, 0, b.desc_bytes);
    // static parts of the instance records
    for (ft_batch::group& g : b.groups)
        for (size_t m = 0; m < g.members.size(); m++) {
            batch_inst* r = (batch_inst*)(b.h_desc + g.off_inst) + m;
            r->prm = (const double*)(g.d_prm + m * g.prm_stride);
            r->tab = g.d_tab + m * g.tab_stride;
        }
    cu(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    cu(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming), "cudaEventCreate");
    cu(cudaEventCreate(&b.ev0), "cudaEventCreate");
    cu(cudaEventCreate(&b.ev1), "cudaEventCreate");
    cu(cudaDeviceSynchronize(), "batch set-up");
}

// the launches of one run, on b.stream (captured into the graph)
void record(ft_batch& b)
{
    cudaStream_t s = b.stream;
    cu(cudaMemcpyAsync(b.d_desc, b.h_desc, b.desc_bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(descriptors)");
    if (b.precision) cu(cudaMemsetAsync(b.d_qacc, 0, b.qacc_words * 8, s), "cudaMemsetAsync");
    const device_state& ds = dev_state();
    b.launches = 0;
    for (ft_batch::group& g : b.groups) {
        cu(ft::launch_batch_item_states(b.d_desc + g.off_prep, (int)g.members.size(), ds.tpow, g.d_itemM,
                                        g.d_item_state, s),
           "batch item states");
        b.launches++;
    }
    cu(cudaEventRecord(b.fork, s), "cudaEventRecord");
    for (ft_batch::group& g : b.groups) {
        cu(cudaStreamWaitEvent(g.stream, b.fork, 0), "cudaStreamWaitEvent");
        const void* inst = b.d_desc + g.off_inst;
        int ninst = (int)g.members.size();
        class_header* hd = (class_header*)(b.d_desc + g.off_hdr);
        const unsigned long long* total = &hd->total_items;
        unsigned long long* counter = &hd->counter;
        unsigned int* qcount = (unsigned int*)&hd->qcount;
        const unsigned long long* item_state = g.d_item_state;
        const unsigned long long* lanepw = g.d_lanepw;
        int lanebits = g.lanebits;
        unsigned long long chunk = g.chunk;
        double* parts = g.d_parts;
        unsigned long long* queue = g.d_queue;
        unsigned int qcap = (unsigned int)g.qcap;
        void* args[] = {&inst, &ninst, &total, &item_state, &lanepw, &lanebits, &chunk, &counter, &parts, &queue,
                        &qcount, &qcap};
        ft::check(ft::drv().LaunchKernel(g.ks->sample, g.grid, 1, 1, g.ks->block, 1, 1, g.ks->smem,
                                         (CUstream)g.stream, args, nullptr),
                  "launch ft_sample_batch");
        b.launches++;
        unsigned long long* qacc = nullptr;
        if (b.precision) {
            qacc = b.d_qacc + g.off_qacc;
            const unsigned long long* cq = g.d_queue;
            const unsigned int* cqc = qcount;
            void* qargs[] = {&inst, &ninst, &cq, &cqc, &qcap, &qacc};
            ft::check(ft::drv().LaunchKernel(g.k64->queue, g.qgrid, 1, 1, g.k64->block, 1, 1, 0,
                                             (CUstream)g.stream, qargs, nullptr),
                      "launch ft_sample_queue_batch");
            b.launches++;
        }
        cu(ft::launch_batch_finalize(inst, ninst, g.d_parts, g.K, qacc, b.d_out + g.off_out, g.stream),
           "batch finalize");
        b.launches++;
        cu(cudaEventRecord(g.done, g.stream), "cudaEventRecord");
        cu(cudaStreamWaitEvent(s, g.done, 0), "cudaStreamWaitEvent");
    }
    cu(cudaMemcpyAsync(b.h_out, b.d_out, b.out_doubles * 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(results)");
    cu(cudaMemcpyAsync(b.h_hdr_out, b.d_desc, b.hdr_bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(counters)");
}

void capture(ft_batch& b)
{
    if (b.exec) {
        cudaGraphExecDestroy(b.exec);
        b.exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    cu(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
        record(b);
    } catch (...) {
        cudaStreamEndCapture(b.stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    cu(cudaStreamEndCapture(b.stream, &graph), "cudaStreamEndCapture");
    const cudaError_t e = cudaGraphInstantiate(&b.exec, graph, 0);
    cudaGraphDestroy(graph);
    cu(e, "cudaGraphInstantiate");
    b.captures++;
}

// grows the item and queue buffers to what the descriptors need; true when it did
bool ensure_capacity(ft_batch& b, const std::vector<size_t>& qwant)
{
    bool grew = false;
    for (size_t gi = 0; gi < b.groups.size(); gi++) {
        ft_batch::group& g = b.groups[gi];
        const size_t items = std::max<size_t>(g.total_items, 1);
        if (items > g.item_cap) {
            const size_t cap = std::max(items, g.item_cap + g.item_cap / 4);
            cudaFree(g.d_item_state);
            cudaFree(g.d_parts);
            g.d_item_state = nullptr;
            g.d_parts = nullptr;
            g.item_cap = 0;
            cu(cudaMalloc(&g.d_item_state, cap * 32), "cudaMalloc(batch item states)");
            cu(cudaMalloc(&g.d_parts, cap * (8 * g.K + 8) * 8), "cudaMalloc(batch item sums)");
            g.item_cap = cap;
            grew = true;
        }
        if (b.precision && qwant[gi] > g.qcap) {
            const size_t cap = std::min<size_t>(std::max(qwant[gi], g.qcap + g.qcap / 4), 0xffffffffull);
            cudaFree(g.d_queue);
            g.d_queue = nullptr;
            g.qcap = 0;
            cu(cudaMalloc(&g.d_queue, cap * 5 * 8), "cudaMalloc(batch FP64 queue)");
            g.qcap = cap;
            grew = true;
        }
    }
    return grew;
}

}  // namespace

extern "C" {

int ft_batch_create(ft_plan* const* plans, int32_t count, int32_t precision, ft_batch** out)
{
    *out = nullptr;
    try {
        if (!plans || count < 1) throw std::invalid_argument("ft_batch_create: no plans");
        if (precision != FT_PRECISION_FP64 && precision != FT_PRECISION_MIXED)
            throw std::invalid_argument("ft_batch_create: unknown precision");
        std::unique_ptr<ft_batch> b(new ft_batch());
        b->plans.assign(plans, plans + count);
        b->precision = precision;
        if (!plans[0]) throw std::invalid_argument("ft_batch_create: NULL plan");
        b->device = plans[0]->device;
        cu(cudaSetDevice(b->device), "cudaSetDevice");
        build(*b);
        *out = b.release();
        return FT_OK;
    } catch (...) {
        return status_of(std::current_exception());
    }
}

void ft_batch_destroy(ft_batch* b) { delete b; }

int ft_batch_run(ft_batch* b, const ft_run_options* opts, ft_result* results)
{
    try {
        if (!b || !opts || !results) throw std::invalid_argument("ft_batch_run: NULL argument");
        std::lock_guard<std::mutex> lock(b->mu);
        auto t0 = std::chrono::steady_clock::now();
        cu(cudaSetDevice(b->device), "cudaSetDevice");
        std::vector<size_t> qwant(b->groups.size(), 0);
        for (size_t gi = 0; gi < b->groups.size(); gi++) {
            ft_batch::group& g = b->groups[gi];
            const unsigned long long per_item = (unsigned long long)g.ks->block * g.chunk;
            unsigned long long next = 0;
            size_t q = 0;
            for (size_t m = 0; m < g.members.size(); m++) {
                const ft_run_options& o = opts[g.members[m]];
                const unsigned long long N = o.num_samples;
                const unsigned long long items = (N + per_item - 1) / per_item;
                if (o.first_sample > ~0ull / (unsigned long long)g.draws)
                    throw std::invalid_argument("ft_batch_run: first_sample too large");
                batch_inst* r = (batch_inst*)(b->h_desc + g.off_inst) + m;
                r->nsamples = N;
                r->first_item = next;
                r->nitems = items;
                item_prep* p = (item_prep*)(b->h_desc + g.off_prep) + m;
                const ft::xstate s = ft::seed_state(o.seed);
                for (int w = 0; w < 4; w++) p->s[w] = s.s[w];
                p->skip = o.first_sample * (unsigned long long)g.draws;
                p->first_item = next;
                p->nitems = items;
                next += items;
                // hand-offs run at ~1e-5 of the samples; a larger share overflows the
                // queue, which then grows and the run repeats once
                q += (size_t)std::min<unsigned long long>(N, N / 1024 + 1024);
            }
            if (next >= (1ull << 36)) throw std::invalid_argument("ft_batch_run: too many work items");
            g.total_items = next;
            class_header* h = (class_header*)(b->h_desc + g.off_hdr);
            h->total_items = next;
            h->counter = 0;
            h->qcount = 0;
            qwant[gi] = q;
        }
        cudaStream_t st = opts[0].stream ? (cudaStream_t)opts[0].stream : b->stream;
        for (int attempt = 0;; attempt++) {
            if (ensure_capacity(*b, qwant) || !b->exec) capture(*b);
            cu(cudaEventRecord(b->ev0, st), "cudaEventRecord");
            cu(cudaGraphLaunch(b->exec, st), "cudaGraphLaunch");
            cu(cudaEventRecord(b->ev1, st), "cudaEventRecord");
            cu(cudaStreamSynchronize(st), "batch run");
            bool overflow = false;
            for (size_t gi = 0; gi < b->groups.size(); gi++) {
                const class_header* h = (const class_header*)((const unsigned char*)b->h_hdr_out + b->groups[gi].off_hdr);
                const unsigned long long qc = h->qcount & 0xffffffffull;
                if (b->precision && qc > b->groups[gi].qcap) {
                    qwant[gi] = (size_t)(qc + qc / 4 + 1024);
                    overflow = true;
                }
            }
            if (!overflow) break;
            if (attempt >= 2) throw std::runtime_error("ft_batch_run: FP64 hand-off queue keeps overflowing");
        }
        float ms = 0;
        cu(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "cudaEventElapsedTime");
        b->last_ms = ms;
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (size_t i = 0; i < b->plans.size(); i++) {
            const ft_batch::group& g = b->groups[b->group_of[i]];
            const double* acc = b->h_out + g.off_out + (size_t)b->slot_of[i] * (8 * g.K + 8);
            std::vector<double> v(acc, acc + 8 * g.K + 8);
            fill_result(b->plans[i]->P, v, &results[i]);
            results[i].kernel_ms = ms;
            results[i].kernel_launches = b->launches;
            results[i].seconds_sampling = secs;
        }
        return FT_OK;
    } catch (...) {
        return status_of(std::current_exception());
    }
}

int ft_batch_get_info(const ft_batch* b, ft_batch_info* info)
{
    if (!b || !info) return FT_ERR_INVALID_ARGUMENT;
    info->num_integrals = (int32_t)b->plans.size();
    info->num_classes = (int32_t)b->groups.size();
    info->graph_captures = b->captures;
    info->kernel_launches = b->launches;
    info->kernel_ms = b->last_ms;
    unsigned long long items = 0, qcap = 0;
    for (const auto& g : b->groups) {
        items += g.total_items;
        qcap += g.qcap;
    }
    info->work_items = items;
    info->fp64_queue_capacity = qcap;
    return FT_OK;
}

int ft_integrate_batch(ft_plan* const* plans, int32_t count, const ft_run_options* opts, ft_result* results)
{
    // one batch per precision present
    for (int prec = 0; prec < 2; prec++) {
        std::vector<ft_plan*> sel;
        std::vector<ft_run_options> so;
        std::vector<int> idx;
        for (int i = 0; i < count; i++)
            if ((opts[i].precision == FT_PRECISION_MIXED ? 1 : 0) == prec) {
                sel.push_back(plans[i]);
                so.push_back(opts[i]);
                idx.push_back(i);
            }
        if (sel.empty()) continue;
        ft_batch* b = nullptr;
        int rc = ft_batch_create(sel.data(), (int32_t)sel.size(), prec, &b);
        if (rc != FT_OK) return rc;
        std::vector<ft_result> rs(sel.size());
        for (size_t k = 0; k < sel.size(); k++) rs[k] = results[idx[k]];
        rc = ft_batch_run(b, so.data(), rs.data());
        ft_batch_destroy(b);
        if (rc != FT_OK) return rc;
        for (size_t k = 0; k < sel.size(); k++) results[idx[k]] = rs[k];
    }
    return FT_OK;
}

}  // extern "C"
