// libhyk runtime: the C ABI of include/hyk.h.
//
// Module creation generates the CUDA source of one ODE system (hyk_codegen.cpp),
// compiles it with NVRTC straight to an sm_103a cubin, loads it through the
// driver API into the device's primary context (the one torch also uses) and
// keeps the kernel handles.  Launch functions marshal the caller's device
// pointers into one by-value parameter block.  No function here allocates
// device memory except module loading; all buffers are the caller's.

#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "hyk.h"
#include "hyk_internal.hpp"

namespace {
// NVTX range over a host-side phase (compile, launch sequence, graph build),
// visible in Nsight Systems / Nsight Compute timelines; costs nothing
// without a tool attached.
struct NvtxRange {
    explicit NvtxRange(const char *name, bool on = true) : on_(on) {
        if (on_) nvtxRangePushA(name);
    }
    ~NvtxRange() {
        if (on_) nvtxRangePop();
    }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;

  private:
    bool on_;
};
}  // namespace

// Generic kernels compiled by nvcc into this library (hyk_generic.cu).
extern "C" int hyk_generic_dense_eval(const double *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld,
                                      const double *dt, double *out, void *stream);
extern "C" int hyk_generic_dense_eval_f32(const float *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes,
                                          uint64_t ld, const float *dt, float *out, void *stream);
extern "C" int hyk_generic_fp64_peak(int device, double millis, double *flops_per_s, char *err, size_t errlen);
extern "C" int hyk_generic_fp32_peak(int device, double millis, double *flops_per_s, char *err, size_t errlen);
extern "C" int hyk_generic_count_finished(const uint32_t *status, uint64_t n_lanes, uint32_t *finished, void *stream);
extern "C" int hyk_generic_dmath(int fn, const double *x, const double *a, double *out, uint64_t n, void *stream);
extern "C" int hyk_noalloc_scratch(int device, void **ptr, size_t *bytes, char *err, size_t errlen);

namespace {

thread_local std::string g_err;

// The CUDA driver is loaded at run time (dlopen), so that the library also
// loads on machines without a GPU driver (build and symbol checks); every
// driver entry point goes through this table.
#define HYK_STR2(x) #x
#define HYK_STR(x) HYK_STR2(x)
#define HYK_DRIVER_FNS(X) X(cuInit) X(cuDeviceGet) X(cuDevicePrimaryCtxRetain) X(cuDeviceGetAttribute) X(cuCtxSetCurrent) X(cuModuleLoadData) X(cuModuleGetFunction) X(cuFuncSetAttribute) X(cuFuncGetAttribute) X(cuOccupancyMaxActiveBlocksPerMultiprocessor) X(cuModuleUnload) X(cuLaunchKernel) X(cuMemsetD32Async) X(cuMemcpyDtoHAsync) X(cuStreamSynchronize) X(cuGetErrorString) X(cuMemAlloc) X(cuMemFree) X(cuGraphCreate) X(cuGraphAddKernelNode) X(cuGraphInstantiate) X(cuGraphLaunch) X(cuGraphExecDestroy) X(cuGraphDestroy) X(cuModuleGetGlobal) X(cuMemcpyHtoD) X(cuMemcpy2DAsync) X(cuMemcpyDtoH) X(cuMemsetD8)

struct DriverApi {
#define HYK_DECL(f) decltype(&::f) f = nullptr;
    HYK_DRIVER_FNS(HYK_DECL)
#undef HYK_DECL
    bool ok = false;
    std::string err;
};

DriverApi &drv() {
    static DriverApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libcuda.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            api.err = std::string("cannot load the CUDA driver (libcuda.so.1): ") + dlerror();
            return;
        }
#define HYK_LOAD(f)                                                             \
    api.f = reinterpret_cast<decltype(&::f)>(dlsym(h, HYK_STR(f)));             \
    if (!api.f) {                                                               \
        api.err = std::string("CUDA driver symbol missing: ") + HYK_STR(f);     \
        return;                                                                 \
    }
        HYK_DRIVER_FNS(HYK_LOAD)
#undef HYK_LOAD
        api.ok = true;
    });
    return api;
}


int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

std::string cu_msg(CUresult r) {
    const char *s = nullptr;
    if (drv().ok) drv().cuGetErrorString(r, &s);
    return s ? s : "unknown CUDA error";
}

#define HYK_CU(call)                                                                                       \
    do {                                                                                                   \
        CUresult hyk_r_ = (call);                                                                          \
        if (hyk_r_ != CUDA_SUCCESS) return fail(HYK_ERR_CUDA, std::string(#call) + ": " + cu_msg(hyk_r_)); \
    } while (0)

// Host mirror of the device parameter block (kernel_template.inc).
struct KParams {
    uint64_t n_lanes, ld;
    double *state;
    const double *pars;
    double *t_hi, *t_lo;
    const double *step_lim;
    double step_default_lim;
    int64_t *step_oc;
    double *step_h;
    double *step_tc;
    const double *tf_hi, *tf_lo, *maxdt;
    uint64_t max_steps;
    const double *grid;
    uint64_t n_grid;
    double *grid_out;
    double *tc_out, *tc_thi, *tc_tlo;
    uint64_t tc_cap;
    double *rem_hi, *rem_lo;
    int64_t *outcome;
    double *min_h, *max_h;
    uint64_t *n_steps, *n_iter, *grid_idx;
    double *last_h, *last_tc;
    uint32_t *status;
    uint64_t iters_per_launch;
    uint64_t *queue;
    uint32_t *finished;
    const uint64_t *lane_order;
    uint64_t n_order;
    const uint32_t *act_count;
    double *ck_x, *ck_t, *ck_h;
    uint64_t ck_cap;
    const int64_t *adj_steps;
    double *adj_lambda, *adj_pbar;
    double *jets;
    double *ev_thi, *ev_tlo;
    int32_t *ev_info;
    uint64_t *ev_cnt;
    uint64_t ev_cap;
    double *ev_last;
    int32_t *ev_sign;
    uint64_t *stop_iter;
    uint64_t stop_group;
    uint64_t *ring;
    uint64_t ring_mask;
    uint64_t *ring_head;
    const uint64_t *ring_tail;
    const uint32_t *serve_stop;
    const int64_t *owner;
    uint32_t *done_count;
    uint64_t *inflight;
    uint32_t *serve_status;
    uint64_t idle_ns, max_wait_ns;
    int persistent;
};

struct Device {
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    int n_sm = 0;
    int smem_optin = 0;   // max dynamic shared memory per block (opt-in)
    int smem_per_sm = 0;  // shared memory per multiprocessor
};

std::mutex g_mtx;
std::map<int, Device> g_devs;
std::map<std::string, std::string> g_cubin_cache;  // key -> cubin bytes

int get_device(int ordinal, Device *&out) {
    if (!drv().ok) return fail(HYK_ERR_CUDA, drv().err);
    std::lock_guard<std::mutex> lk(g_mtx);
    auto it = g_devs.find(ordinal);
    if (it == g_devs.end()) {
        HYK_CU(drv().cuInit(0));
        Device d;
        HYK_CU(drv().cuDeviceGet(&d.dev, ordinal));
        HYK_CU(drv().cuDevicePrimaryCtxRetain(&d.ctx, d.dev));
        HYK_CU(drv().cuDeviceGetAttribute(&d.n_sm, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, d.dev));
        HYK_CU(drv().cuDeviceGetAttribute(&d.smem_optin, CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_BLOCK_OPTIN, d.dev));
        HYK_CU(drv().cuDeviceGetAttribute(&d.smem_per_sm, CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_MULTIPROCESSOR, d.dev));
        int major = 0, minor = 0;
        HYK_CU(drv().cuDeviceGetAttribute(&major, CU_DEVICE_ATTRIBUTE_COMPUTE_CAPABILITY_MAJOR, d.dev));
        HYK_CU(drv().cuDeviceGetAttribute(&minor, CU_DEVICE_ATTRIBUTE_COMPUTE_CAPABILITY_MINOR, d.dev));
        if (major != 10 || minor != 3)
            return fail(HYK_ERR_UNSUPPORTED, "libhyk targets sm_103 (GB300); device " + std::to_string(ordinal) +
                                                 " is sm_" + std::to_string(major) + std::to_string(minor));
        it = g_devs.emplace(ordinal, d).first;
    }
    out = &it->second;
    HYK_CU(drv().cuCtxSetCurrent(out->ctx));
    return 0;
}

uint64_t fnv1a(const std::string &s, uint64_t h = 1469598103934665603ULL) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ULL;
    }
    return h;
}

std::string cache_dir() {
    const char *e = std::getenv("HYK_CACHE_DIR");
    if (e && *e) return e;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/hyk";
}

int compile_nvrtc(const std::string &src, const std::string &name, std::string &cubin, std::string &log) {
    NvtxRange nv("hyk: NVRTC compile");
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), name.c_str(), 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) return fail(HYK_ERR_NVRTC, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    std::vector<const char *> opts = {"--gpu-architecture=sm_103a", "--fmad=false", "-std=c++17", "-lineinfo",
                                      "--restrict"};
    const char *pv = std::getenv("HYK_PTXAS_VERBOSE");
    if (pv && *pv == '1') opts.push_back("--ptxas-options=-v");
    r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    log.assign(ls, '\0');
    if (ls) nvrtcGetProgramLog(prog, &log[0]);
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return fail(HYK_ERR_NVRTC, "NVRTC compilation failed: " + log);
    }
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    cubin.assign(cs, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return 0;
}

}  // namespace

struct hyk_module {
    hyk::Dec d;
    uint32_t order = 0;
    hyk_config_t cfg{};
    int device = 0;
    Device *dv = nullptr;
    CUmodule mod = nullptr;
    CUfunction f_step = nullptr, f_prop = nullptr, f_init = nullptr, f_adj = nullptr;
    CUfunction f_azero = nullptr, f_alist = nullptr;  // the plain form's list of unfinished lanes
    CUfunction f_serve = nullptr;                     // the serving kernel (lane form)
    int adj_ctas_per_sm = 0;
    uint32_t team = 0;           // threads per trajectory (team form); 0 = lane form
    bool f32 = false;            // single precision
    bool gmem = false;           // Taylor coefficients in a global buffer (large systems)
    uint64_t gmem_threads = 0;   // threads of the fixed grid in that mode
    uint32_t ncold = 0;          // cold state rows in the global buffer (0: none)
    uint64_t cold_threads = 0;   // threads of the fixed grid the cold rows are sized for
    int cold_ctas = 0;           // CTAs per SM of that grid
    CUdeviceptr jets = 0;        // the module's coefficient buffer (gmem mode)
    std::string src, log;
    uint32_t blk = 0, nslot = 0;
    size_t smem = 0;
    int regs = 0, local_bytes = 0, ctas_per_sm = 0;
    double flops = 0, compile_s = 0;

    // Releases the loaded code and the coefficient buffer (also on the error
    // paths of hyk_module_create).
    ~hyk_module() {
        if (!mod && !jets) return;
        if (dv) drv().cuCtxSetCurrent(dv->ctx);
        if (jets) drv().cuMemFree(jets);
        if (mod) drv().cuModuleUnload(mod);
    }
};

extern "C" {

const char *hyk_last_error(void) { return g_err.c_str(); }
const char *hyk_version(void) { return "hyk 0.1 (sm_103a, FP64 and FP32 Taylor, NVRTC)"; }

int hyk_module_create(const hyk_decomp_t *dd, uint32_t order, const hyk_config_t *cfg, int device, hyk_module **out) {
    NvtxRange nv("hyk: module create");
    if (!out) return fail(HYK_ERR_INVALID, "null output pointer");
    *out = nullptr;
    std::unique_ptr<hyk_module> m(new hyk_module());
    std::string err;
    if (!hyk::load_dec(dd, m->d, err)) return fail(HYK_ERR_INVALID, err);
    if (order < 2 || order > 200) return fail(HYK_ERR_INVALID, "the Taylor order must be in [2, 200]");
    if (cfg) m->cfg = *cfg;
    m->order = order;
    m->device = device;
    const bool adjoint = (m->cfg.flags & HYK_CFG_ADJOINT) != 0;
    const bool pin = (m->cfg.flags & HYK_CFG_PIN_ARITH) != 0;
    const bool f32 = (m->cfg.flags & HYK_CFG_FLOAT32) != 0;
    if (f32 && (pin || adjoint))
        return fail(HYK_ERR_UNSUPPORTED, "single precision supports neither pin arithmetic nor the adjoint");
    m->f32 = f32;
    int rc = get_device(device, m->dv);
    if (rc) return rc;
    const Device &dv = *m->dv;

    const size_t real_bytes = f32 ? sizeof(float) : sizeof(double);
    uint32_t nslot = hyk::count_slots(m->d, order, adjoint, pin);
    size_t lane_bytes = (size_t)nslot * real_bytes;
    uint32_t blk = m->cfg.block_lanes;

    // Form.  The lane form (one thread per trajectory) needs 32 lanes of
    // coefficients per warp in shared memory and at least 4 resident warps
    // per SM to keep the four FP64 pipes busy.  The team form spreads one
    // trajectory over 2..32 threads: smaller shared memory per warp, at the
    // price of idle threads in the rounds of each dependency level.  The
    // estimate compares busy-thread share x min(1, warps per SM / 4).
    hyk::TeamInfo ti;
    std::string terr;
    const bool team_ok = !adjoint && !pin && hyk::team_layout(m->d, order, ti, terr);
    const uint32_t want_team = m->cfg.team_size;
    if (want_team > 32 || (want_team & (want_team - 1)))
        return fail(HYK_ERR_INVALID, "team_size must be 0, 1 or a power of two up to 32");
    if (want_team > 1) {
        if (!team_ok)
            return fail(HYK_ERR_UNSUPPORTED, std::string("the team form is not available: ") +
                                                 (adjoint ? "adjoint module" : pin ? "pin arithmetic" : terr));
        m->team = want_team;
    } else if (want_team == 0 && team_ok) {
        // Lane form: shared memory with w warps per SM scores min(1, w / 4);
        // global-memory coefficients (eight warps per SM) score 0.7 (measured:
        // CR3BP 52 % of the FP64 peak against Kepler's 62 % from shared memory).
        const size_t warp_bytes = 32 * lane_bytes;
        double best = 0.7;
        if (warp_bytes <= (size_t)dv.smem_optin) {
            const double w = (double)((size_t)dv.smem_per_sm / (warp_bytes + 1024));
            best = std::max(best, std::min(1.0, w / 4.0));
        }
        for (uint32_t T = 2, l = 1; T <= 32; T *= 2, ++l) {
            const size_t cta = (size_t)(32 / T) * ti.n_slot * real_bytes;
            if (cta > (size_t)dv.smem_optin) continue;
            const double w = (double)((size_t)dv.smem_per_sm / (cta + 1024));
            const double score = ti.util[l] * std::min(1.0, w / 4.0) * 0.85;
            if (score > best) {
                best = score;
                m->team = T;
            }
        }
    }
    if (m->team) {
        if (blk == 0) blk = 32;
        nslot = ti.n_slot;
        lane_bytes = (size_t)nslot * real_bytes;
    }
    // Lane form of a system whose coefficients do not fit 32 lanes of shared
    // memory: a global buffer owned by the module, one slot stride for the
    // whole fixed grid, so a warp still reads 32 consecutive doubles.
    //
    // Also when shared memory would hold fewer than four warps per SM (or the
    // caller asks for it): the global-memory form runs eight warps per SM,
    // and each of the four FP64 pipes of an SM needs a ready warp of its own
    // (CR3BP: 3 warps from shared memory 42 % of the FP64 peak, global 52 %).
    const size_t smem_warps = (size_t)dv.smem_per_sm / (lane_bytes * 32 + 1024);
    m->gmem = !m->team && (lane_bytes * 32 > (size_t)dv.smem_optin || smem_warps < 4 ||
                           (m->cfg.flags & HYK_CFG_GLOBAL_JETS) != 0);
    // Team form with its coefficient regions in global memory (on request):
    // one region per team of a fixed resident grid, few enough to stay in L2,
    // so more warps per SM than shared memory holds.
    if (m->team && (m->cfg.flags & HYK_CFG_GLOBAL_JETS) != 0) m->gmem = true;
    if (m->team) {
        // one CTA per warp by default: finest packing of the shared memory;
        // with global-memory regions four warps per CTA
        if (m->gmem && blk == 0) blk = 128;
        // Cold state rows (every state variable read at its current order
        // only: the N-body problem): two shared-memory slots per state
        // variable instead of p + 1, its orders in a global buffer of the
        // module; taken when that fits more CTAs on an SM (the 6-body
        // problem at order 19: 1593 slots instead of 2277, eight CTAs of two
        // trajectories instead of six).
        if (!m->gmem && ti.n_slot_cold && !(m->cfg.flags & HYK_CFG_NO_COLD_ROWS)) {
            const size_t tpc = blk / m->team;
            const size_t hot = tpc * ti.n_slot * real_bytes, cold = tpc * ti.n_slot_cold * real_bytes;
            const uint32_t ch = hot > (size_t)dv.smem_optin ? 0 : (uint32_t)((size_t)dv.smem_per_sm / (hot + 1024));
            const uint32_t cc = cold > (size_t)dv.smem_optin ? 0 : (uint32_t)((size_t)dv.smem_per_sm / (cold + 1024));
            if (std::min<uint32_t>(cc, 32) > std::min<uint32_t>(ch, 32)) {
                nslot = ti.n_slot_cold;
                lane_bytes = (size_t)nslot * real_bytes;
                m->ncold = m->d.n_eq;
                m->cold_ctas = (int)std::min<uint32_t>(cc, 32);
                m->cold_threads = (uint64_t)dv.n_sm * (uint64_t)m->cold_ctas * blk;
            }
        }
    } else if (m->gmem) {
        // The recurrences as one function per order (no spills), with their
        // own slots for the order-0 reciprocals.
        nslot = hyk::count_slots(m->d, order, adjoint, pin, false, nullptr, true);
        lane_bytes = (size_t)nslot * real_bytes;
        // Two CTAs of 128 threads per SM by default: at most 255 registers a
        // thread, so both fit the register file, and eight warps hide the
        // latency of the global-memory coefficients better than four.
        if (blk == 0) blk = 128;
        const uint32_t ctas = m->cfg.persist_ctas ? m->cfg.persist_ctas : (blk <= 128 ? 2 : 1);
        m->gmem_threads = (uint64_t)dv.n_sm * ctas * blk;
    } else {
        // Pick the block size maximising resident lanes per SM under the
        // shared-memory budget (1 KiB per CTA is reserved by the hardware),
        // capped at 256 per CTA and at 512 lanes per SM in double precision
        // (the FP64 pipe saturates with far fewer warps) or 768 in single
        // precision (more warps hide the dependent-issue latency of the
        // FP32 pipe).
        // The double-precision lane kernels use (nearly) all 255 registers a
        // thread can have, so at most 256 threads share an SM's 64K registers.
        const uint32_t lane_cap = f32 ? 768u : 512u;
        const uint32_t reg_threads = f32 ? 1024u : 256u;
        auto pick = [&](size_t lbytes, uint32_t &b_out, uint32_t &lanes_out) {
            b_out = 0;
            lanes_out = 0;
            for (uint32_t b = 32; b <= 256; b += 32) {
                const size_t per_cta = b * lbytes;
                if (per_cta > (size_t)dv.smem_optin) break;
                uint32_t ctas = (uint32_t)((size_t)dv.smem_per_sm / (per_cta + 1024));
                ctas = std::min(ctas, reg_threads / b);
                uint32_t lanes = std::min<uint32_t>(ctas * b, lane_cap);
                if (lanes >= lanes_out) {
                    lanes_out = lanes;
                    b_out = b;
                }
            }
        };
        uint32_t best = 0, best_lanes = 0;
        pick(lane_bytes, best, best_lanes);
        // Cold state rows: when the state variables that no recurrence reads
        // at a later order move their orders 1..p to a global buffer of the
        // module, more lanes may fit (Kepler at order 19: 99 slots instead of
        // 156, eight warps per SM instead of five).  A sub-partition with a
        // single warp leaves its FP64 pipe idle while that warp waits on
        // shared-memory loads and other latencies; two warps keep it busy.
        uint32_t ncold = 0;
        const uint32_t cslots = adjoint || !m->d.ev.empty() || (m->cfg.flags & HYK_CFG_NO_COLD_ROWS)
                                    ? nslot
                                    : hyk::count_slots(m->d, order, adjoint, pin, true, &ncold);
        if (ncold > 0 && cslots < nslot) {
            uint32_t cb = 0, clanes = 0;
            pick((size_t)cslots * real_bytes, cb, clanes);
            if (blk) {  // the caller's block size: cold rows whenever they fit more of its CTAs
                const size_t hot = (size_t)blk * nslot * real_bytes, cold = (size_t)blk * cslots * real_bytes;
                const uint32_t ch = hot > (size_t)dv.smem_optin ? 0 : (uint32_t)((size_t)dv.smem_per_sm / (hot + 1024));
                const uint32_t cc = cold > (size_t)dv.smem_optin ? 0 : (uint32_t)((size_t)dv.smem_per_sm / (cold + 1024));
                cb = blk;
                clanes = std::min(cc, reg_threads / blk) > std::min(ch, reg_threads / blk) ? std::min(cc, reg_threads / blk) * blk : 0;
                best_lanes = 0;
            }
            if (clanes > best_lanes && clanes >= 32 * 4) {
                best = cb;
                best_lanes = clanes;
                nslot = cslots;
                lane_bytes = (size_t)nslot * real_bytes;
                m->ncold = ncold;
                m->cold_ctas = (int)std::min<size_t>((size_t)dv.smem_per_sm / ((size_t)cb * lane_bytes + 1024),
                                                     reg_threads / cb);
                m->cold_threads = (uint64_t)dv.n_sm * (uint64_t)m->cold_ctas * cb;
            }
        }
        if (blk == 0) {
            if (best == 0) {
                if (lane_bytes * 32 > (size_t)dv.smem_optin)
                    return fail(HYK_ERR_UNSUPPORTED, "the system needs " + std::to_string(lane_bytes) +
                                                         " bytes of Taylor coefficients per lane; at most " +
                                                         std::to_string(dv.smem_optin / 32) + " fit the shared memory");
                best = 32;
            }
            blk = best;
        }
    }
    if (blk % 32 != 0 || blk > 1024) return fail(HYK_ERR_INVALID, "block_lanes must be a multiple of 32, <= 1024");
    m->blk = blk;
    m->nslot = nslot;
    m->smem = m->gmem ? 0 : m->team ? (size_t)(blk / m->team) * lane_bytes : (size_t)blk * lane_bytes;
    if (m->smem > (size_t)dv.smem_optin)
        return fail(HYK_ERR_UNSUPPORTED, "shared memory per CTA (" + std::to_string(m->smem) + ") exceeds the device limit");

    hyk::GenOut g;
    const bool high_acc = (m->cfg.flags & HYK_CFG_HIGH_ACCURACY) != 0;
    if (m->team) {
        if (!hyk::generate_team(m->d, order, m->team, blk, sizeof(KParams), g, err, high_acc, f32, m->gmem, m->ncold != 0))
            return fail(HYK_ERR_INVALID, err);
    } else if (!hyk::generate(m->d, order, pin, blk, sizeof(KParams), g, err, adjoint, m->gmem ? m->gmem_threads : 0,
                              high_acc, f32, m->ncold ? m->cold_threads : 0, m->gmem)) {
        return fail(HYK_ERR_INVALID, err);
    }
    if (g.n_slot != nslot || g.n_cold != m->ncold) return fail(HYK_ERR_INVALID, "internal: slot count mismatch");
    m->src = (m->cfg.flags & HYK_CFG_DEBUG) ? "#define HYK_DEBUG 1\n" + g.src : g.src;
    m->flops = g.flops;

    const auto t0 = std::chrono::steady_clock::now();
    const std::string key = std::to_string(fnv1a(m->src)) + "_sm103a";
    std::string cubin;
    {
        std::lock_guard<std::mutex> lk(g_mtx);
        auto it = g_cubin_cache.find(key);
        if (it != g_cubin_cache.end()) cubin = it->second;
    }
    const std::string dpath = cache_dir() + "/" + key + ".cubin";
    if (cubin.empty() && !std::getenv("HYK_NO_DISK_CACHE")) {
        std::ifstream f(dpath, std::ios::binary);
        if (f) {
            std::ostringstream ss;
            ss << f.rdbuf();
            cubin = ss.str();
        }
    }
    if (cubin.empty()) {
        rc = compile_nvrtc(m->src, "hyk_module.cu", cubin, m->log);
        if (rc) return rc;
        if (!std::getenv("HYK_NO_DISK_CACHE")) {
            std::string cmd = "mkdir -p '" + cache_dir() + "'";
            if (std::system(cmd.c_str()) == 0) {
                std::ofstream f(dpath + ".tmp", std::ios::binary);
                f.write(cubin.data(), (std::streamsize)cubin.size());
                f.close();
                std::rename((dpath + ".tmp").c_str(), dpath.c_str());
            }
        }
    }
    {
        std::lock_guard<std::mutex> lk(g_mtx);
        g_cubin_cache[key] = cubin;
    }
    m->compile_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    HYK_CU(drv().cuModuleLoadData(&m->mod, cubin.data()));
    if (m->gmem && !m->team) HYK_CU(drv().cuMemAlloc(&m->jets, (size_t)m->gmem_threads * lane_bytes));
    if (m->ncold) {
        // The cold rows' buffer and its address in the module's constant
        // hyk_cold_base (read by every kernel thread of the module).
        // (lane form: orders 1..p of each cold row per thread; team form:
        // orders 0..p of every state variable per team)
        const size_t cold_bytes = m->team ? (size_t)(m->cold_threads / m->team) * m->ncold * (order + 1) * real_bytes
                                          : (size_t)m->cold_threads * m->ncold * order * real_bytes;
        HYK_CU(drv().cuMemAlloc(&m->jets, cold_bytes));
        CUdeviceptr cb = 0;
        size_t cbytes = 0;
        HYK_CU(drv().cuModuleGetGlobal(&cb, &cbytes, m->mod, "hyk_cold_base"));
        if (cbytes != sizeof(CUdeviceptr)) return fail(HYK_ERR_INVALID, "internal: hyk_cold_base size");
        HYK_CU(drv().cuMemcpyHtoD(cb, &m->jets, sizeof(CUdeviceptr)));
    }
    HYK_CU(drv().cuModuleGetFunction(&m->f_step, m->mod, "hyk_step_kernel"));
    HYK_CU(drv().cuModuleGetFunction(&m->f_prop, m->mod, "hyk_prop_kernel"));
    HYK_CU(drv().cuModuleGetFunction(&m->f_init, m->mod, "hyk_prop_init_kernel"));
    HYK_CU(drv().cuModuleGetFunction(&m->f_azero, m->mod, "hyk_act_zero_kernel"));
    HYK_CU(drv().cuModuleGetFunction(&m->f_alist, m->mod, "hyk_act_list_kernel"));
    if (!m->team) {
        HYK_CU(drv().cuModuleGetFunction(&m->f_serve, m->mod, "hyk_serve_kernel"));
        HYK_CU(drv().cuFuncSetAttribute(m->f_serve, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)m->smem));
        HYK_CU(drv().cuFuncSetAttribute(m->f_serve, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT,
                                        m->gmem ? 0 : 100));
    }
    for (CUfunction f : {m->f_step, m->f_prop}) {
        HYK_CU(drv().cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)m->smem));
        // Global-memory coefficients: no shared memory, the whole unified
        // on-chip array as L1 to cache them.
        HYK_CU(drv().cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, m->gmem ? 0 : 100));
    }
    HYK_CU(drv().cuFuncGetAttribute(&m->regs, CU_FUNC_ATTRIBUTE_NUM_REGS, m->f_prop));
    HYK_CU(drv().cuFuncGetAttribute(&m->local_bytes, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, m->f_prop));
    HYK_CU(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&m->ctas_per_sm, m->f_prop, (int)blk, m->smem));
    if (m->gmem && m->team) {
        // CTAs per SM: the occupancy limit, at most as many as keep the
        // teams' regions within 100 MB (of the 126 MB L2), or the caller's
        // persist_ctas
        const uint64_t cta_bytes = (uint64_t)(blk / m->team) * lane_bytes;
        const int by_l2 = (int)std::max<uint64_t>(1, (100ull << 20) / (cta_bytes * (uint64_t)dv.n_sm));
        int c = std::min(m->ctas_per_sm, by_l2);
        if (m->cfg.persist_ctas) {
            if ((int)m->cfg.persist_ctas > m->ctas_per_sm)
                return fail(HYK_ERR_UNSUPPORTED, "persist_ctas exceeds the CTAs that can be resident on an SM");
            c = (int)m->cfg.persist_ctas;
        }
        if (c < 1) return fail(HYK_ERR_UNSUPPORTED, "the propagation kernel cannot be resident on an SM");
        m->ctas_per_sm = c;
        m->gmem_threads = (uint64_t)dv.n_sm * c * blk;
        HYK_CU(drv().cuMemAlloc(&m->jets, (size_t)dv.n_sm * c * cta_bytes));
    } else if (m->gmem) {
        const int want = (int)(m->gmem_threads / ((uint64_t)dv.n_sm * blk));
        if (m->ctas_per_sm < want) return fail(HYK_ERR_UNSUPPORTED, "the global-memory grid cannot be resident");
        m->ctas_per_sm = want;
    } else if (m->ncold) {
        // Launches never exceed the grid the cold rows are sized for.
        m->ctas_per_sm = std::min(m->ctas_per_sm, m->cold_ctas);
    }
    if (adjoint) {
        HYK_CU(drv().cuModuleGetFunction(&m->f_adj, m->mod, "hyk_adjoint_kernel"));
        HYK_CU(drv().cuFuncSetAttribute(m->f_adj, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)m->smem));
        HYK_CU(drv().cuFuncSetAttribute(m->f_adj, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT,
                                        m->gmem ? 0 : 100));
        HYK_CU(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&m->adj_ctas_per_sm, m->f_adj, (int)blk, m->smem));
        if (m->adj_ctas_per_sm < 1) return fail(HYK_ERR_UNSUPPORTED, "the adjoint kernel cannot be resident on an SM");
        if (m->gmem) {
            if (m->adj_ctas_per_sm < m->ctas_per_sm)
                return fail(HYK_ERR_UNSUPPORTED, "the global-memory adjoint grid cannot be resident");
            m->adj_ctas_per_sm = m->ctas_per_sm;
        }
    }
    if (m->ctas_per_sm < 1) return fail(HYK_ERR_UNSUPPORTED, "the propagation kernel cannot be resident on an SM");
    *out = m.release();
    return 0;
}

int hyk_module_destroy(hyk_module *m) {
    delete m;  // the destructor unloads the module and frees its buffer
    return 0;
}

int hyk_module_get_info(const hyk_module *m, hyk_module_info_t *info) {
    if (!m || !info) return fail(HYK_ERR_INVALID, "null argument");
    std::memset(info, 0, sizeof *info);
    info->n_eq = m->d.n_eq;
    info->n_pars = m->d.n_pars;
    info->order = m->order;
    info->n_u = m->d.n_u();
    info->block_lanes = m->blk;
    info->smem_per_lane = m->gmem ? 0u : m->nslot * (m->f32 ? 4u : 8u);
    info->team_size = m->team ? m->team : 1;
    info->regs_per_thread = (uint32_t)m->regs;
    info->ctas_per_sm = (uint32_t)m->ctas_per_sm;
    info->n_sm = (uint32_t)m->dv->n_sm;
    info->reserved = (uint32_t)m->local_bytes;
    info->flops_per_step = m->flops;
    info->compile_seconds = m->compile_s;
    return 0;
}

const char *hyk_module_source(const hyk_module *m) { return m ? m->src.c_str() : ""; }

int hyk_module_debug(hyk_module *m, uint64_t out[8], int clear) {
    if (!m || !out) return fail(HYK_ERR_INVALID, "null argument");
    if (!(m->cfg.flags & HYK_CFG_DEBUG)) return fail(HYK_ERR_INVALID, "the module was not created with HYK_CFG_DEBUG");
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    CUdeviceptr rec = 0;
    size_t bytes = 0;
    HYK_CU(drv().cuModuleGetGlobal(&rec, &bytes, m->mod, "hyk_dbg"));
    if (bytes != 8 * sizeof(uint64_t)) return fail(HYK_ERR_INVALID, "internal: hyk_dbg size");
    HYK_CU(drv().cuMemcpyDtoH(out, rec, bytes));
    if (clear) HYK_CU(drv().cuMemsetD8(rec, 0, bytes));
    return 0;
}

static int check_lanes(const hyk_module *m, const hyk_lanes_t *l) {
    if (!m || !l) return fail(HYK_ERR_INVALID, "null argument");
    if (l->n_lanes == 0) return 0;
    if (l->ld < l->n_lanes) return fail(HYK_ERR_INVALID, "ld must be >= n_lanes");
    if (!l->state || !l->time_hi || !l->time_lo) return fail(HYK_ERR_INVALID, "null state or time pointer");
    if (m->d.n_pars && !l->pars) return fail(HYK_ERR_INVALID, "the system has parameters but pars is NULL");
    return 0;
}

static void fill_lanes(KParams &k, const hyk_lanes_t *l) {
    std::memset(&k, 0, sizeof k);
    k.n_lanes = l->n_lanes;
    k.ld = l->ld;
    k.state = l->state;
    k.pars = l->pars;
    k.t_hi = l->time_hi;
    k.t_lo = l->time_lo;
}

// Blocks covering n trajectories: blk of them per block in the lane form,
// blk / team in the team form.
static uint64_t lane_blocks(const hyk_module *m, uint64_t n) {
    const uint64_t per = m->team ? m->blk / m->team : m->blk;
    return (n + per - 1) / per;
}

// Grid of a launch of f: in global-memory mode every kernel but the
// initialisation runs on the fixed grid the coefficient buffer is sized for.
static uint64_t launch_grid(const hyk_module *m, CUfunction f, uint64_t grid) {
    if ((m->gmem || m->ncold) && f != m->f_init) grid = std::min<uint64_t>(grid, (uint64_t)m->dv->n_sm * m->ctas_per_sm);
    return grid;
}

static int launch(hyk_module *m, CUfunction f, uint64_t grid, uint32_t blk, size_t smem, KParams &k, void *stream) {
    if (grid == 0) return 0;
    k.jets = reinterpret_cast<double *>(m->jets);
    grid = launch_grid(m, f, grid);
    if (grid > 0x7fffffffULL) return fail(HYK_ERR_INVALID, "too many lanes for one launch");
    void *args[] = {&k};
    HYK_CU(drv().cuLaunchKernel(f, (unsigned)grid, 1, 1, blk, 1, 1, (unsigned)smem, (CUstream)stream, args, nullptr));
    return 0;
}

// A CUDA graph of a chain of launches with the same parameter block (the
// plain propagation's launches between two reads of the unfinished-lane
// count).  The parameter block is copied into the nodes.
struct LaunchGraph {
    CUgraph g = nullptr;
    CUgraphExec x = nullptr;
    ~LaunchGraph() {
        if (x) drv().cuGraphExecDestroy(x);
        if (g) drv().cuGraphDestroy(g);
    }
};

struct LaunchSpec {
    CUfunction f;
    uint64_t grid;
    uint32_t blk;
    size_t smem;
};

// The launches of one round of the plain propagation after the round's first
// listing: with a lane list, [step, (zero, list, step) x (per_round - 1)];
// without one, per_round step launches.  Generated on demand (no container),
// so the direct-launch path keeps no heap storage.
struct PlainRound {
    bool compact;
    uint32_t per_round;
    uint64_t grid, lgrid;
    uint32_t size() const { return compact ? 1 + 3 * (per_round - 1) : per_round; }
    LaunchSpec at(const hyk_module *m, uint32_t i) const {
        if (compact && i > 0) {
            switch ((i - 1) % 3) {
            case 0:
                return {m->f_azero, 1, 32, 0};
            case 1:
                return {m->f_alist, lgrid, 256, 0};
            default:
                break;
            }
        }
        return {m->f_prop, grid, m->blk, m->smem};
    }
};

static int build_graph(hyk_module *m, const PlainRound &round, KParams &k, LaunchGraph &lg) {
    NvtxRange nv("hyk: build step graph");
    k.jets = reinterpret_cast<double *>(m->jets);
    HYK_CU(drv().cuGraphCreate(&lg.g, 0));
    void *args[] = {&k};
    CUgraphNode prev = nullptr;
    for (uint32_t i = 0; i < round.size(); ++i) {
        const LaunchSpec ls = round.at(m, i);
        const uint64_t grid = launch_grid(m, ls.f, ls.grid);
        if (grid == 0 || grid > 0x7fffffffULL) return fail(HYK_ERR_INVALID, "too many lanes for one launch");
        CUDA_KERNEL_NODE_PARAMS np;
        std::memset(&np, 0, sizeof np);
        np.func = ls.f;
        np.gridDimX = (unsigned)grid;
        np.gridDimY = np.gridDimZ = 1;
        np.blockDimX = ls.blk;
        np.blockDimY = np.blockDimZ = 1;
        np.sharedMemBytes = (unsigned)ls.smem;
        np.kernelParams = args;
        CUgraphNode node;
        HYK_CU(drv().cuGraphAddKernelNode(&node, lg.g, prev ? &prev : nullptr, prev ? 1 : 0, &np));
        prev = node;
    }
    HYK_CU(drv().cuGraphInstantiate(&lg.x, lg.g, 0));
    return 0;
}

// Event buffers of a module with events (all of them are required then).
static int fill_events(const hyk_module *m, KParams &k, const hyk_prop_t *p) {
    if (m->d.ev.empty()) return 0;
    if (!p || !p->ev_t_hi || !p->ev_t_lo || !p->ev_info || !p->ev_count || !p->ev_last || !p->ev_sign)
        return fail(HYK_ERR_INVALID, "a module with events needs the event buffers (ev_t_hi, ev_t_lo, ev_info, "
                                     "ev_count, ev_last, ev_sign)");
    k.ev_thi = p->ev_t_hi;
    k.ev_tlo = p->ev_t_lo;
    k.ev_info = p->ev_info;
    k.ev_cnt = p->ev_count;
    k.ev_cap = p->ev_capacity;
    k.ev_last = p->ev_last;
    k.ev_sign = p->ev_sign;
    return 0;
}

int hyk_step(hyk_module *m, const hyk_lanes_t *lanes, const double *max_delta_t, int backward, int64_t *outcome,
             double *h, double *tc, const struct hyk_prop *ev, void *stream) {
    NvtxRange nv("hyk: step");
    int rc = check_lanes(m, lanes);
    if (rc) return rc;
    if (!outcome || !h) return fail(HYK_ERR_INVALID, "null outcome or h pointer");
    if (lanes->n_lanes == 0) return 0;
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    KParams k;
    fill_lanes(k, lanes);
    rc = fill_events(m, k, ev);
    if (rc) return rc;
    k.step_lim = max_delta_t;
    k.step_default_lim = backward ? -INFINITY : INFINITY;
    k.step_oc = outcome;
    k.step_h = h;
    k.step_tc = tc;
    return launch(m, m->f_step, lane_blocks(m, lanes->n_lanes), m->blk, m->smem, k, stream);
}

static int fill_prop(hyk_module *m, KParams &k, const hyk_lanes_t *lanes, const hyk_prop_t *p) {
    if (!p) return fail(HYK_ERR_INVALID, "null propagation descriptor");
    if (!p->tf_hi || !p->rem_hi || !p->rem_lo || !p->outcome || !p->min_h || !p->max_h || !p->n_steps ||
        !p->n_iter || !p->status || !p->last_h)
        return fail(HYK_ERR_INVALID, "a required propagation array is NULL");
    if (p->grid && (!p->grid_out || !p->grid_idx || p->n_grid == 0))
        return fail(HYK_ERR_INVALID, "grid propagation needs grid_out, grid_idx and n_grid >= 1");
    if (p->tc_out && (!p->tc_t_hi || !p->tc_t_lo))
        return fail(HYK_ERR_INVALID, "Taylor-coefficient capture needs tc_t_hi and tc_t_lo");
    fill_lanes(k, lanes);
    k.tf_hi = p->tf_hi;
    k.tf_lo = p->tf_lo;
    k.maxdt = p->max_delta_t;
    k.max_steps = p->max_steps;
    k.grid = p->grid;
    k.n_grid = p->n_grid;
    k.grid_out = p->grid_out;
    k.tc_out = p->tc_out;
    k.tc_thi = p->tc_t_hi;
    k.tc_tlo = p->tc_t_lo;
    k.tc_cap = p->tc_capacity;
    k.rem_hi = p->rem_hi;
    k.rem_lo = p->rem_lo;
    k.outcome = p->outcome;
    k.min_h = p->min_h;
    k.max_h = p->max_h;
    k.n_steps = p->n_steps;
    k.n_iter = p->n_iter;
    k.grid_idx = p->grid_idx;
    k.last_h = p->last_h;
    k.last_tc = p->last_tc;
    k.status = p->status;
    k.lane_order = p->lane_order;
    k.n_order = p->lane_order ? p->n_order : lanes->n_lanes;
    k.ck_x = p->ck_x;
    k.ck_t = p->ck_t;
    k.ck_h = p->ck_h;
    k.ck_cap = p->ck_capacity;
    if (p->ck_x && (!p->ck_t || !p->ck_h)) return fail(HYK_ERR_INVALID, "the checkpoint tape needs ck_x, ck_t and ck_h");
    k.stop_iter = p->stop_iter;
    k.stop_group = p->stop_group;
    return fill_events(m, k, p);
}

int hyk_prop_init(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, void *stream) {
    int rc = check_lanes(m, lanes);
    if (rc) return rc;
    if (lanes->n_lanes == 0) return 0;
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    KParams k;
    rc = fill_prop(m, k, lanes, p);
    if (rc) return rc;
    return launch(m, m->f_init, (lanes->n_lanes + 127) / 128, 128, 0, k, stream);
}

// Counters: the queue (8 B at 0), the finished-lane count (4 B at 8) and the
// active-lane count (4 B at 12), padded to 256 B.  The plain form also takes,
// after them, the list of unfinished lanes (8 B per lane); with a workspace
// of only the counters it steps the lanes in place instead.
static constexpr size_t kWsCounters = 256;

static bool plain_compacts(const hyk_module *m, uint64_t n_lanes, size_t workspace_bytes) {
    return m && n_lanes > 0 && workspace_bytes >= kWsCounters + 8 * n_lanes;
}

size_t hyk_propagate_workspace_size(const hyk_module *m, uint64_t n_lanes, int mode) {
    if (mode == HYK_MODE_PLAIN && m) return kWsCounters + 8 * n_lanes;
    return kWsCounters;
}

// hyk_propagate and hyk_propagate_noalloc.  use_graphs: the plain form
// replays its rounds as a CUDA graph (hyk_propagate); without it every
// launch is made directly, so that nothing is created or instantiated
// (hyk_propagate_noalloc, whose callers must not allocate).
static int propagate_impl(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, int mode, void *workspace,
                          size_t workspace_bytes, uint32_t check_every, uint64_t *iters, void *stream, bool use_graphs) {
    // (no NVTX call on the no-allocation path: a tool's NVTX handler may allocate)
    NvtxRange nv(mode == HYK_MODE_PERSISTENT ? "hyk: propagate (persistent)" : "hyk: propagate (plain)", use_graphs);
    int rc = check_lanes(m, lanes);
    if (rc) return rc;
    if (iters) *iters = 0;
    if (lanes->n_lanes == 0) return 0;
    if (!workspace || workspace_bytes < kWsCounters) return fail(HYK_ERR_INVALID, "workspace too small");
    if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return fail(HYK_ERR_INVALID, "workspace must be 256-byte aligned");
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    KParams k;
    rc = fill_prop(m, k, lanes, p);
    if (rc) return rc;
    k.queue = reinterpret_cast<uint64_t *>(workspace);
    k.finished = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(workspace) + 8);
    const CUstream s = (CUstream)stream;
    if (mode == HYK_MODE_PERSISTENT) {
        HYK_CU(drv().cuMemsetD32Async((CUdeviceptr)workspace, 0, 4, s));
        k.persistent = 1;
        k.iters_per_launch = p->slice_iters ? p->slice_iters : ~0ULL;
        // The resident capacity, whatever the number of lanes: a CTA that
        // finds the queue empty returns at once, and spreading a small batch
        // over every SM gives each of its warps an FP64 unit of its own.
        const uint64_t grid = (uint64_t)m->dv->n_sm * (uint64_t)m->ctas_per_sm;
        rc = launch(m, m->f_prop, grid, m->blk, m->smem, k, stream);
        if (rc) return rc;
        if (iters) *iters = 1;
        return 0;
    }
    if (mode != HYK_MODE_PLAIN) return fail(HYK_ERR_INVALID, "unknown propagation mode");
    // One launch per step, in rounds of check_every launches; between rounds
    // one word is read back (the only host synchronisation of the loop).
    // With room for the lane list, every step launch is preceded by two small
    // launches that list the unfinished lanes (hyk_act_zero_kernel,
    // hyk_act_list_kernel), and the step launch steps only those (a grid of
    // at most the resident capacity looping over the list, whose length it
    // reads from device memory), so warps are not left half idle by lanes
    // that finished; the word read back is the list's length.  Without it,
    // every launch covers all lanes and the word is the number of finished
    // lanes.  With use_graphs, from the second round on a round's launches are
    // one CUDA graph (built once per call and replayed: the launch parameters
    // do not change); otherwise every launch is made directly.
    if (check_every == 0) check_every = 16;
    k.persistent = 0;
    k.iters_per_launch = 1;
    const bool compact = plain_compacts(m, lanes->n_lanes, workspace_bytes);
    uint64_t grid = lane_blocks(m, lanes->n_lanes);
    PlainRound chain{compact, check_every, grid, std::min<uint64_t>(4096, (lanes->n_lanes + 255) / 256)};
    if (compact) {
        k.lane_order = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(workspace) + kWsCounters);
        k.n_order = 0;
        k.act_count = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(workspace) + 12);
        chain.grid = std::min<uint64_t>(grid, (uint64_t)m->dv->n_sm * (uint64_t)m->ctas_per_sm);
    } else {
        rc = hyk_generic_count_finished(p->status, lanes->n_lanes, k.finished, stream);
        if (rc) return rc;
    }
    uint64_t n = 0;
    uint32_t word = 0;
    const bool graphs = use_graphs && check_every > 1;
    LaunchGraph lg;
    for (uint64_t r = 0;; ++r) {
        if (compact) {
            rc = launch(m, m->f_azero, 1, 32, 0, k, stream);
            if (!rc) rc = launch(m, m->f_alist, chain.lgrid, 256, 0, k, stream);
            if (rc) return rc;
            HYK_CU(drv().cuMemcpyDtoHAsync(&word, (CUdeviceptr)k.act_count, sizeof word, s));
            HYK_CU(drv().cuStreamSynchronize(s));
            if (word == 0) break;
        } else {
            HYK_CU(drv().cuMemcpyDtoHAsync(&word, (CUdeviceptr)k.finished, sizeof word, s));
            HYK_CU(drv().cuStreamSynchronize(s));
            if ((uint64_t)word >= lanes->n_lanes) break;
        }
        if (graphs && r >= 1) {
            if (!lg.x) {
                rc = build_graph(m, chain, k, lg);
                if (rc) return rc;
            }
            HYK_CU(drv().cuGraphLaunch(lg.x, s));
            n += check_every;
            continue;
        }
        for (uint32_t i = 0; i < chain.size(); ++i) {
            const LaunchSpec ls = chain.at(m, i);
            rc = launch(m, ls.f, ls.grid, ls.blk, ls.smem, k, stream);
            if (rc) return rc;
            if (ls.f == m->f_prop) ++n;
        }
    }
    if (iters) *iters = n;
    return 0;
}

int hyk_propagate(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, int mode, void *workspace,
                  size_t workspace_bytes, uint32_t check_every, uint64_t *iters, void *stream) {
    return propagate_impl(m, lanes, p, mode, workspace, workspace_bytes, check_every, iters, stream, true);
}

// Propagation without a caller workspace: the counters hyk_propagate keeps in
// its workspace come from libhyk's file-scope device scratch array
// (hyk_noalloc.cu).  Nothing here allocates: the scratch address is looked up
// once per device, the counters are cleared at the start of every call, and
// the plain form launches every kernel directly (no CUDA graph is created or
// instantiated, no host container is filled).
int hyk_propagate_noalloc(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, int mode, uint32_t check_every,
                          uint64_t *iters, void *stream) {
    if (!m) return fail(HYK_ERR_INVALID, "null module");
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    void *ws = nullptr;
    size_t cap = 0;
    char buf[256] = {0};
    if (hyk_noalloc_scratch(m->device, &ws, &cap, buf, sizeof buf)) return fail(HYK_ERR_CUDA, buf);
    // The counters always fit; the plain form's lane list does when the
    // batch is small enough, and the plain form steps the lanes in place
    // otherwise.
    if (kWsCounters > cap) return fail(HYK_ERR_INVALID, "hyk_propagate_noalloc: the scratch array is too small");
    return propagate_impl(m, lanes, p, mode, ws, cap, check_every, iters, stream, false);
}

int hyk_serve(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, const hyk_serve_t *sv, void *stream) {
    NvtxRange nv("hyk: serve launch");
    int rc = check_lanes(m, lanes);
    if (rc) return rc;
    if (!m->f_serve) return fail(HYK_ERR_UNSUPPORTED, "serving with a device work queue needs a lane-form module");
    if (!sv || !sv->ring || !sv->head || !sv->tail || !sv->stop || !sv->owner || !sv->done_count || !sv->inflight ||
        !sv->status)
        return fail(HYK_ERR_INVALID, "null serving-queue pointer");
    if (sv->ring_capacity == 0 || (sv->ring_capacity & (sv->ring_capacity - 1)))
        return fail(HYK_ERR_INVALID, "the ring capacity must be a power of two");
    if (sv->max_wait_ns == 0) return fail(HYK_ERR_INVALID, "max_wait_ns must be positive (every wait is bounded)");
    if (lanes->n_lanes == 0) return 0;
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    KParams k;
    rc = fill_prop(m, k, lanes, p);
    if (rc) return rc;
    if (k.grid || k.tc_out || k.ck_x || !m->d.ev.empty())
        return fail(HYK_ERR_UNSUPPORTED, "the serving kernel propagates without grids, coefficient output, tapes or events");
    k.persistent = 1;
    k.iters_per_launch = ~0ULL;
    k.ring = sv->ring;
    k.ring_mask = sv->ring_capacity - 1;
    k.ring_head = sv->head;
    k.ring_tail = sv->tail;
    k.serve_stop = sv->stop;
    k.owner = sv->owner;
    k.done_count = sv->done_count;
    k.inflight = sv->inflight;
    k.serve_status = sv->status;
    k.idle_ns = sv->idle_ns;
    k.max_wait_ns = sv->max_wait_ns;
    uint64_t grid = (uint64_t)m->dv->n_sm * (uint64_t)m->ctas_per_sm;
    if (sv->grid_ctas) grid = std::min<uint64_t>(grid, sv->grid_ctas);
    return launch(m, m->f_serve, grid, m->blk, m->smem, k, stream);
}

int hyk_memcpy2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height, void *stream) {
    if (width == 0 || height == 0) return 0;
    if (!dst || !src || dpitch < width || spitch < width) return fail(HYK_ERR_INVALID, "invalid 2D copy");
    CUDA_MEMCPY2D c;
    std::memset(&c, 0, sizeof c);
    c.srcMemoryType = CU_MEMORYTYPE_UNIFIED;
    c.srcDevice = (CUdeviceptr)src;
    c.srcPitch = spitch;
    c.dstMemoryType = CU_MEMORYTYPE_UNIFIED;
    c.dstDevice = (CUdeviceptr)dst;
    c.dstPitch = dpitch;
    c.WidthInBytes = width;
    c.Height = height;
    HYK_CU(drv().cuMemcpy2DAsync(&c, (CUstream)stream));
    return 0;
}

int hyk_adjoint(hyk_module *m, const hyk_lanes_t *lanes, const double *ck_x, const double *ck_t, const double *ck_h,
                const int64_t *n_steps, const uint64_t *lane_order, double *lambda, double *pbar, void *workspace,
                size_t workspace_bytes, void *stream) {
    NvtxRange nv("hyk: adjoint");
    int rc = check_lanes(m, lanes);
    if (rc) return rc;
    if (!m->f_adj) return fail(HYK_ERR_INVALID, "the module was not created with HYK_CFG_ADJOINT");
    if (lanes->n_lanes == 0) return 0;
    if (!ck_x || !ck_t || !ck_h || !n_steps || !lambda || (m->d.n_pars && !pbar))
        return fail(HYK_ERR_INVALID, "null tape, step-count, adjoint or parameter-adjoint pointer");
    if (!workspace || workspace_bytes < 256 || (reinterpret_cast<uintptr_t>(workspace) & 255u))
        return fail(HYK_ERR_INVALID, "the workspace must be at least 256 bytes, 256-byte aligned");
    HYK_CU(drv().cuCtxSetCurrent(m->dv->ctx));
    KParams k;
    fill_lanes(k, lanes);
    k.ck_x = const_cast<double *>(ck_x);
    k.ck_t = const_cast<double *>(ck_t);
    k.ck_h = const_cast<double *>(ck_h);
    k.ck_cap = (uint64_t)INT64_MAX;  // the caller's tape holds n_steps[lane] steps for every lane
    k.adj_steps = n_steps;
    k.lane_order = lane_order;
    k.adj_lambda = lambda;
    k.adj_pbar = pbar;
    k.queue = reinterpret_cast<uint64_t *>(workspace);
    const CUstream s = (CUstream)stream;
    HYK_CU(drv().cuMemsetD32Async((CUdeviceptr)workspace, 0, 2, s));
    const uint64_t grid = (uint64_t)m->dv->n_sm * (uint64_t)m->adj_ctas_per_sm;
    return launch(m, m->f_adj, grid, m->blk, m->smem, k, stream);
}

int hyk_dense_eval(const double *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld, const double *dt,
                   double *out, void *stream) {
    if (n_lanes == 0) return 0;
    if (!tc || !dt || !out || ld < n_lanes || n_eq == 0) return fail(HYK_ERR_INVALID, "invalid dense-output arguments");
    const int rc = hyk_generic_dense_eval(tc, n_eq, order, n_lanes, ld, dt, out, stream);
    if (rc) return fail(HYK_ERR_CUDA, "dense-output kernel launch failed");
    return 0;
}

int hyk_dense_eval_f32(const float *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld, const float *dt,
                       float *out, void *stream) {
    if (n_lanes == 0) return 0;
    if (!tc || !dt || !out || ld < n_lanes || n_eq == 0) return fail(HYK_ERR_INVALID, "invalid dense-output arguments");
    const int rc = hyk_generic_dense_eval_f32(tc, n_eq, order, n_lanes, ld, dt, out, stream);
    if (rc) return fail(HYK_ERR_CUDA, "dense-output kernel launch failed");
    return 0;
}

int hyk_codegen_check(const hyk_decomp_t *dd, uint32_t order, const hyk_config_t *cfg, int verbose, char *log,
                      size_t log_len, uint32_t *n_slot, double *flops) {
    hyk::Dec d;
    std::string err;
    if (!hyk::load_dec(dd, d, err)) return fail(HYK_ERR_INVALID, err);
    if (order < 2 || order > 200) return fail(HYK_ERR_INVALID, "the Taylor order must be in [2, 200]");
    const uint32_t blk = (cfg && cfg->block_lanes) ? cfg->block_lanes : 128;
    const bool pin = cfg && (cfg->flags & HYK_CFG_PIN_ARITH);
    const bool adjoint = cfg && (cfg->flags & HYK_CFG_ADJOINT);
    // The same choice as the runtime: coefficients in global memory when 32
    // lanes do not fit the opt-in shared memory of an SM (227 KB), with the
    // slot stride of a 152-SM grid.
    const uint32_t team = cfg ? cfg->team_size : 0;
    const bool f32 = cfg && (cfg->flags & HYK_CFG_FLOAT32);
    if (verbose == 4) {  // recurrences for the compiled CPU stepper (reference arithmetic, any element type)
        std::string hs;
        if (!hyk::generate_host_batch(d, order, hs, err)) return fail(HYK_ERR_UNSUPPORTED, err);
        if (hs.size() + 1 > log_len || !log) return fail(HYK_ERR_INVALID, "log buffer too small for the generated source");
        std::snprintf(log, log_len, "%s", hs.c_str());
        return 0;
    }
    if (team > 1 && verbose == 3) {  // host translation unit of the team form
        std::string hs;
        const bool cold = !(cfg->flags & HYK_CFG_NO_COLD_ROWS) && !(cfg->flags & HYK_CFG_GLOBAL_JETS);
        if (!hyk::generate_host(d, order, false, hs, err, true, f32, cold)) return fail(HYK_ERR_UNSUPPORTED, err);
        if (log && log_len) std::snprintf(log, log_len, "%s", hs.c_str());
        return 0;
    }
    const uint32_t slots = hyk::count_slots(d, order, adjoint, pin);
    // The global-memory layout when 32 lanes do not fit shared memory or on
    // request (HYK_CFG_GLOBAL_JETS), with the slot stride of two CTAs per SM.
    const bool want_g = (uint64_t)slots * (f32 ? 4 : 8) * 32 > 227u * 1024 || (cfg && (cfg->flags & HYK_CFG_GLOBAL_JETS));
    const uint64_t gstride = want_g ? 2ull * 152ull * blk : 0;
    // The cold-state-row layout (as the runtime may pick it), with the rows
    // sized for one CTA per SM of a 152-SM GPU.
    uint32_t ncold = 0;
    if (!gstride && !adjoint && d.ev.empty() && !(cfg && (cfg->flags & HYK_CFG_NO_COLD_ROWS)))
        hyk::count_slots(d, order, adjoint, pin, true, &ncold);
    const uint64_t cstride = ncold ? 152ull * blk : 0;
    hyk::GenOut g;
    const bool high_acc = cfg && (cfg->flags & HYK_CFG_HIGH_ACCURACY);
    if (team > 1) {
        const bool tg = (cfg->flags & HYK_CFG_GLOBAL_JETS) != 0;
        if (!hyk::generate_team(d, order, team, cfg->block_lanes ? cfg->block_lanes : (tg ? 128 : 32), sizeof(KParams),
                                g, err, high_acc, f32, tg, !(cfg->flags & HYK_CFG_NO_COLD_ROWS)))
            return fail(HYK_ERR_UNSUPPORTED, err);
    } else if (!hyk::generate(d, order, pin, blk, sizeof(KParams), g, err, adjoint, gstride, high_acc, f32, cstride,
                              gstride != 0)) {
        return fail(HYK_ERR_INVALID, err);
    }
    if (n_slot) *n_slot = g.n_slot;
    if (flops) *flops = g.flops;
    if (verbose == 3) {  // host translation unit (CPU checks of the generator)
        std::string hs;
        if (!hyk::generate_host(d, order, adjoint, hs, err, false, f32)) return fail(HYK_ERR_INVALID, err);
        if (log && log_len) std::snprintf(log, log_len, "%s", hs.c_str());
        return 0;
    }
    if (verbose == 2) {  // source only, no compilation
        if (log && log_len) std::snprintf(log, log_len, "%s", g.src.c_str());
        return 0;
    }
    if (cfg && (cfg->flags & HYK_CFG_DEBUG)) g.src = "#define HYK_DEBUG 1\n" + g.src;
    if (verbose) setenv("HYK_PTXAS_VERBOSE", "1", 1);
    std::string cubin, lg;
    const int rc = compile_nvrtc(g.src, "hyk_check.cu", cubin, lg);
    if (verbose) unsetenv("HYK_PTXAS_VERBOSE");
    if (log && log_len) {
        std::snprintf(log, log_len, "%s", lg.c_str());
    }
    return rc;
}

int hyk_dmath_eval(int fn, const double *x, const double *a, double *out, uint64_t n, void *stream) {
    if (fn < 0 || fn > 11) return fail(HYK_ERR_INVALID, "unknown function index");
    if (n && (!x || !out || ((fn == 4 || fn == 5 || fn == 10 || fn == 11) && !a)))
        return fail(HYK_ERR_INVALID, "null argument");
    if (hyk_generic_dmath(fn, x, a, out, n, stream)) return fail(HYK_ERR_CUDA, "dmath kernel launch failed");
    return 0;
}

int hyk_fp64_peak(int device, double millis, double *flops_per_s) {
    char buf[256] = {0};
    const int rc = hyk_generic_fp64_peak(device, millis, flops_per_s, buf, sizeof buf);
    if (rc) return fail(HYK_ERR_CUDA, buf);
    return 0;
}

int hyk_fp32_peak(int device, double millis, double *flops_per_s) {
    char buf[256] = {0};
    const int rc = hyk_generic_fp32_peak(device, millis, flops_per_s, buf, sizeof buf);
    if (rc) return fail(HYK_ERR_CUDA, buf);
    return 0;
}

}  // extern "C"

// Compile-time check that the module source carries the same parameter block.
static_assert(sizeof(KParams) % 8 == 0, "unexpected KParams padding");
