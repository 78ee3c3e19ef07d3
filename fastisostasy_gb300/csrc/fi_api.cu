// fi_api.cu — host side of the C ABI declared in include/fi_gpu.h.
//
// One fi_handle = one padded LV-ELVA domain resident on the current CUDA
// device, with its own stream.  The host code restates the init-time logic
// of isos_init's method-3 branch (src/fastisostasy.f90:64-473) and drives
// the device kernels in the order of isos_update
// (src/fastisostasy.f90:731-872).  There is no CPU compute path: every
// per-cell operation of init_state/update runs on the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <functional>
#include <mutex>
#include <condition_variable>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/fi_gpu.h"
#include "fi_engine.h"
#include "fi_init.h"
#include "fi_kernels.h"
#include "fi_batch.h"
#include "fi_state.h"

using namespace fi;

namespace {

// Host API ranges for timeline tools (NVTX: inert unless a tool is attached)
// and the host-time accounting of the update calls.
struct ApiRange {
    explicit ApiRange(const char* name) { nvtxRangePushA(name); }
    ~ApiRange() { nvtxRangePop(); }
};
struct UpdateClock {
    fi_handle* h;
    std::chrono::steady_clock::time_point t0;
    explicit UpdateClock(fi_handle* hh);
    ~UpdateClock();
};

}  // namespace

namespace {

// A small persistent pool of host threads for the copies between the
// caller's arrays and the page-locked staging buffer (a single core copies a
// few GB/s; the isos%out fields are ~100 B per cell).  run(n, fn) calls
// fn(0..n-1) on the workers and the calling thread and returns when all are
// done; one job at a time.
class HostPool {
public:
    static HostPool& get()
    {
        static HostPool p;
        return p;
    }
    void run(int ntasks, const std::function<void(int)>& fn)
    {
        if (ntasks <= 1 || workers_.empty()) {
            for (int i = 0; i < ntasks; ++i) fn(i);
            return;
        }
        std::lock_guard<std::mutex> job(job_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &fn;
            ntasks_ = ntasks;
            next_ = 0;
            pending_ = ntasks;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return pending_ == 0; });
        fn_ = nullptr;
    }

private:
    HostPool()
    {
        unsigned hw = std::thread::hardware_concurrency();
        const int nw = (int)std::min<unsigned>(hw > 1 ? hw - 1 : 0, 15u);
        for (int i = 0; i < nw; ++i)
            workers_.emplace_back([this] {
                unsigned long long seen = 0;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> lk(mu_);
                        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                        if (stop_) return;
                        seen = gen_;
                    }
                    work();
                }
            });
    }
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    void work()
    {
        for (;;) {
            int i;
            const std::function<void(int)>* f;
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!fn_ || next_ >= ntasks_) return;
                i = next_++;
                f = fn_;
            }
            (*f)(i);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_cv_.notify_all();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex mu_, job_mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* fn_ = nullptr;
    int ntasks_ = 0, next_ = 0, pending_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

// dst <- src in `parts` slices on the pool
// A caller buffer in page-locked host memory (cudaHostAlloc, or a range
// registered with cudaHostRegister) is copied to and from the device
// directly; pageable memory goes through the handle's staging buffer.
bool host_pinned(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void pool_copy(void* dst, const void* src, size_t bytes, int parts)
{
    const size_t chunk = (bytes + parts - 1) / parts;
    HostPool::get().run(parts, [&](int i) {
        const size_t a = (size_t)i * chunk;
        if (a < bytes) memcpy((char*)dst + a, (const char*)src + a, std::min(chunk, bytes - a));
    });
}


const double PI_LIT = (double)3.14159265359f;   // src/isostasy_defs.f90:8 (default-real literal)
inline double sp(double x) { return (double)(float)x; }

FftDesc factorize(int n)
{
    FftDesc d;
    memset(&d, 0, sizeof(d));
    d.n = n;
    int m = n, e2 = 0;
    while (m % 2 == 0) { m /= 2; e2++; }
    int n8 = e2 / 3, r = e2 % 3, n4 = 0, n2 = 0;
    if (r == 1) { if (n8 > 0) { n8--; n4 = 2; } else n2 = 1; }
    else if (r == 2) n4 = 1;
    for (int i = 0; i < n8; ++i) d.fac[d.nf++] = 8;
    for (int i = 0; i < n4; ++i) d.fac[d.nf++] = 4;
    for (int i = 0; i < n2; ++i) d.fac[d.nf++] = 2;
    for (int f = 3; m > 1; f += 2)
        while (m % f == 0) { d.fac[d.nf++] = f; m /= f; }
    return d;
}

bool nice(int n)
{
    for (int f : {2, 3, 5, 7})
        while (n % f == 0) n /= f;
    return n == 1;
}
int nice_even_at_least(int m)
{
    int v = m + (m & 1);
    while (!nice(v)) v += 2;
    return v;
}

// The 42-entry table of get_ge_value (src/green_functions.f90:56-66,
// 131-168), interpolated on the device; the radii are multiplied by 1.e3 in
// single precision there.
const float kRn[42] = {0.0f, 0.011f, 0.111f, 1.112f, 2.224f, 3.336f, 4.448f, 6.672f, 8.896f, 11.12f, 17.79f,
                       22.24f, 27.80f, 33.36f, 44.48f, 55.60f, 66.72f, 88.96f, 111.2f, 133.4f, 177.9f, 222.4f,
                       278.0f, 333.6f, 444.8f, 556.0f, 667.2f, 778.4f, 889.6f, 1001.0f, 1112.0f, 1334.0f,
                       1779.0f, 2224.0f, 2780.0f, 3336.0f, 4448.0f, 5560.0f, 6672.0f, 7784.0f, 8896.0f, 10008.0f};
const float kGe[42] = {-33.6488f, -33.64f, -33.56f, -32.75f, -31.86f, -30.98f, -30.12f, -28.44f, -26.87f,
                       -25.41f, -21.80f, -20.02f, -18.36f, -17.18f, -15.71f, -14.91f, -14.41f, -13.69f, -13.01f,
                       -12.31f, -10.95f, -9.757f, -8.519f, -7.533f, -6.131f, -5.237f, -4.660f, -4.272f, -3.999f,
                       -3.798f, -3.640f, -3.392f, -2.999f, -2.619f, -2.103f, -1.530f, -0.292f, 0.848f, 1.676f,
                       2.083f, 2.057f, 1.643f};


}  // namespace

struct fi_handle {
    fi_params p;
    int nx, ny, nx_ice, ny_ice, icrop1, icrop2, jcrop1, jcrop2;
    size_t n;
    double dx, dy, spy, cc, Vden;
    int init_rc = 0;                   // device init of kappa, GE, GN
    double rate_scale = 1.0;           // stage outputs -> rates: sec/yr (method 3) or 1 (methods 0-2)
    double L_w = 0.0;                  // flexural length scale (LV-ELRA)
    double time_diag, time_prog;
    int ref_was_set = 0, state_ready = 0;
    double h_t = 0.0, h_dt = 0.0;       // host mirror of the ode clock (euler/rk4)
    double ref_bsl = 0.0;
    int Px = 0, Py = 0;
    int even = 1, uniform = 1;
    long long launches = 0;            // kernels enqueued by this handle
    long long updates = 0;             // isos_update calls (fi_update, fi_update_async)
    double host_update_s = 0.0;        // host time spent inside them (enqueue + copies + waits)
    // CUDA graphs of whole updates, keyed by (step count, diagnostics, ...)
    struct GraphEntry {
        long long key;
        long long nkernels;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs;
    std::vector<long long> graph_seen;
    bool use_graphs = true;
    bool tsit_graph_ok = true;         // Tsit5 attempts loop on the device inside captured graphs
    bool require_tsit_graph = false;   // FI_REQUIRE_TSIT_GRAPH=1: no host-loop fallback (tests)
    // persistent cooperative RK4 engine (true stages, uniform spacing)
    bool engine_ok = false;
    int eng_grid = 0, eng_CB = 1, eng_RA = 2, eng_P2 = 0;
    size_t eng_smem = 0;
    float *xhi = nullptr, *xlo = nullptr, *wrefhi = nullptr, *wreflo = nullptr;
    float* dxw = nullptr;   // (xhi - wrefhi) + (xlo - wreflo): the kernel sequence's mixed RK4 stages
    // true-stage Tsit5, mixed form: the stage state as a float pair and its dxw
    float *yhi = nullptr, *ylo = nullptr, *ydw = nullptr;
    unsigned long long* trace = nullptr;   // engine phase timestamps (fi_engine_trace)
    // optional per-kernel CUDA-event timing (fi_profile)
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_ev;
    std::vector<int> prof_id;
    size_t prof_used = 0;
    double prof_ms[32] = {0};
    long long prof_cnt[32] = {0};
    cudaStream_t s = nullptr;            // work of this handle (its own, or the caller's: fi_set_stream)
    cudaStream_t s_own = nullptr;        // the handle's own stream while the caller's is in use
    cudaStream_t s_body = nullptr;       // captures the body of the device Tsit5 loop
    std::vector<void*> allocs;
    std::string err;
    cudaError_t launch_err = cudaSuccess;   // a launch whose status the enqueue path cannot return
    // fi_update's output path: one event per staged field and a page-locked
    // copy of the control block, so the host unpacks a field while the
    // later ones are still being copied
    std::vector<cudaEvent_t> ev_field;
    Ctl* hctl = nullptr;
    // host copies of the static fields
    std::vector<double> K, kappa, R, D, He, eta_eff, GE, GN, GV, xc, yc;
    std::vector<uint8_t> mact;
    // device
    Dom d;
    Ctl* ctl = nullptr;
    Plan2D prhs, pconv;
    Plan2D pconv_run;   // pconv with the transform shapes tuned for the update's precision
    FlexCoef fc;
    double* y = nullptr;                 // stage state
    void* q0 = nullptr;                  // RHS load term (T)
    void* Dt = nullptr;                  // rigidity (T)
    void* inv2eta = nullptr;             // 1/(2 eta_eff) (T)
    void* f = nullptr;                   // flexure output (T)
    void* raw[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // RHS stage outputs (T)
    int* dmore = nullptr;                // loop condition of the eager true-stage Tsit5 path
    void* S = nullptr;                   // RHS half spectrum (T complex)
    void* mA = nullptr;                  // 1/(kappa R) at (k, l) (T)
    void* mB = nullptr;                  // 1/(kappa R) at (-k, l) (T)
    // step engine only: the half spectrum and the factors column-major
    // (element (l, k) at k*ny + l), so a spectrum column is contiguous
    void* ST = nullptr;
    unsigned* eng_bar = nullptr;   // the step engine's grid-barrier counter
    // page-locked status of the caller's host arrays seen by fi_update (the
    // same arrays come back every step; a stale entry only costs speed:
    // cudaMemcpyAsync from pageable memory is still correct)
    struct PinSeen {
        const void* p;
        bool pinned;
    } pin_seen[16] = {};
    int pin_next = 0;
    void* mAT = nullptr;
    void* mBT = nullptr;
    void* S2 = nullptr;                  // convolution spectrum (T complex)
    void* KS[3] = {nullptr, nullptr, nullptr};   // elastic / geoid / LV-ELRA viscous kernel spectra (T complex)
    double* weq = nullptr;               // equilibrium displacement (methods 0-2)
    double* weq_raw = nullptr;           // LV-ELRA convolution output
    void* conv_in = nullptr;             // convolution input (T)
    double *we_raw = nullptr, *dz_raw = nullptr, *corners = nullptr;
    int* out_rows = nullptr;
    double* dH = nullptr;                // ice-grid thickness on the device
    double* dpack = nullptr;             // packed outputs
    double* dsnap = nullptr;             // asynchronous output: device snapshot (11 x ice grid)
    cudaStream_t s_out = nullptr;        // asynchronous output: copy stream
    cudaEvent_t ev_snap = nullptr, ev_out = nullptr;
    bool out_pending = false;
    double* hpin = nullptr;              // pinned staging (max(ice grid, packed outputs))
    size_t hpin_elems = 0;
    const double** gsrc = nullptr;
    const uint8_t** gmsrc = nullptr;
    double *dxm = nullptr, *dym = nullptr;
    // reference-state device pointers (non-const views)
    double *z_bed_ref, *Hice_ref, *Haf_ref, *z_ss_ref, *we_ref, *w_ref, *dz_ss_ref;
    uint8_t *mo_ref, *mg_ref, *mc_ref;
};

namespace {

int fail(fi_handle* h, int code, const char* fmt, ...)
{
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) return fail(h, FI_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// Kernel ids of the profiler (fi_profile_read): see include/fi_gpu.h.
enum { K_FLEX = 0, K_ROWS_FWD, K_COLS_HARTLEY, K_ROWS_INV, K_CONV_ROWS_FWD, K_CONV_COLS, K_CONV_ROWS_INV,
       K_STAGE, K_RK_FINAL, K_UPD_BEGIN, K_UPD_MASKS, K_UPD_LITHO, K_UPD_LOAD, K_UPD_END, K_CONTROL, K_TS,
       K_ENGINE, K_NPROF };

int prof_begin(fi_handle* h, int id)
{
    if (!h->prof_on) return -1;
    if (h->prof_used + 2 > h->prof_ev.size()) {
        const size_t add = 4096;
        for (size_t i = 0; i < add; ++i) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            h->prof_ev.push_back(e);
        }
        h->prof_id.resize(h->prof_ev.size() / 2 + 1);
    }
    const int m = (int)h->prof_used;
    cudaEventRecord(h->prof_ev[m], h->s);
    h->prof_id[m / 2] = id;
    h->prof_used += 2;
    return m;
}
void prof_end(fi_handle* h, int m)
{
    if (m >= 0) cudaEventRecord(h->prof_ev[m + 1], h->s);
}
void prof_collect(fi_handle* h)
{
    if (h->prof_used == 0) return;
    cudaStreamSynchronize(h->s);
    for (size_t m = 0; m + 1 < h->prof_used; m += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h->prof_ev[m], h->prof_ev[m + 1]) == cudaSuccess) {
            h->prof_ms[h->prof_id[m / 2]] += ms;
            h->prof_cnt[h->prof_id[m / 2]] += 1;
        }
    }
    h->prof_used = 0;
}
#define PROF(h, id, expr)                  \
    do {                                   \
        const int pm_ = prof_begin(h, id); \
        expr;                              \
        prof_end(h, pm_);                  \
    } while (0)

template <typename P> int dalloc(fi_handle* h, P** out, size_t bytes)
{
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    // stream-ordered on the handle's stream: creating and destroying handles
    // (a serving loop) never synchronises the device under other requests
    cudaError_t e = cudaMallocAsync(&p, bytes, h->s);
    if (e != cudaSuccess) {
        *out = nullptr;
        return fail(h, e == cudaErrorMemoryAllocation ? FI_E_OOM : FI_E_CUDA, "cudaMallocAsync(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    h->allocs.push_back(p);
    cudaMemsetAsync(p, 0, bytes, h->s);
    *out = static_cast<P*>(p);
    return FI_OK;
}

bool mixed(const fi_handle* h) { return h->p.precision == FI_PREC_MIXED; }
size_t tsz(const fi_handle* h) { return mixed(h) ? sizeof(float) : sizeof(double); }

int upload(fi_handle* h, void* dst, const void* src, size_t bytes)
{
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->s));
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

// double host vector -> device buffer of the field type
int upload_T(fi_handle* h, void* dst, const std::vector<double>& v)
{
    if (mixed(h)) {
        std::vector<float> t(v.size());
        for (size_t i = 0; i < v.size(); ++i) t[i] = (float)v[i];
        return upload(h, dst, t.data(), t.size() * sizeof(float));
    }
    return upload(h, dst, v.data(), v.size() * sizeof(double));
}

int make_len(fi_handle* h, int n, FftLen& L)
{
    L.d = factorize(n);
    std::vector<double2> t64(n);
    std::vector<float2> t32(n);
    for (int t = 0; t < n; ++t) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
        t64[t] = make_double2((double)cosl(a), (double)sinl(a));
        t32[t] = make_float2((float)cosl(a), (float)sinl(a));
    }
    double2* d64;
    float2* d32;
    int rc;
    if ((rc = dalloc(h, &d64, n * sizeof(double2))) || (rc = dalloc(h, &d32, n * sizeof(float2)))) return rc;
    if ((rc = upload(h, d64, t64.data(), n * sizeof(double2))) || (rc = upload(h, d32, t32.data(), n * sizeof(float2))))
        return rc;
    L.tw64 = d64;
    L.tw32 = d32;
    return FI_OK;
}

int make_plan(fi_handle* h, int nx, int ny, Plan2D& P)
{
    P.nx = nx;
    P.ny = ny;
    P.h = nx / 2;
    P.sp = ((P.h + 1) + 7) / 8 * 8;
    int rc;
    if ((rc = make_len(h, P.h, P.row)) || (rc = make_len(h, ny, P.col))) return rc;
    std::vector<double2> r64(P.h + 1);
    std::vector<float2> r32(P.h + 1);
    for (int k = 0; k <= P.h; ++k) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)nx;
        r64[k] = make_double2((double)cosl(a), (double)sinl(a));
        r32[k] = make_float2((float)cosl(a), (float)sinl(a));
    }
    double2* d64;
    float2* d32;
    if ((rc = dalloc(h, &d64, (P.h + 1) * sizeof(double2))) || (rc = dalloc(h, &d32, (P.h + 1) * sizeof(float2))))
        return rc;
    if ((rc = upload(h, d64, r64.data(), (P.h + 1) * sizeof(double2))) ||
        (rc = upload(h, d32, r32.data(), (P.h + 1) * sizeof(float2))))
        return rc;
    P.rtw64 = d64;
    P.rtw32 = d32;
    return FI_OK;
}

// ---- init-time physics (host, double) ---------------------------------------
double rigidity(double E, double He, double nu) { return E * 1e9 * (He * He * He) / (12.0 * (1.0 - nu * nu)); }

// Kelvin function kei for LV-ELRA.  The reference interpolates a table of
// kei(x) at x = 0, 0.01, .., 10 printed with five significant digits and
// stored as single-precision literals (src/kelvin_function.f90:91-132,
// 166-1233).  The table is computed here from the function itself,
// kei(x) = Im K_0(x e^{i pi/4}) = -int_0^inf exp(-a) sin(a) dt with
// a = x cosh(t) / sqrt(2) (trapezoid rule on an even analytic integrand),
// then rounded the same way.
double kelvin_kei(double x)
{
    if (x <= 0.0) return -0.78539816339744830962;   // -pi/4
    const double h = 1.0 / 64.0, r2 = std::sqrt(2.0);
    double sum = 0.0;
    for (int k = 0;; ++k) {
        const double a = x * std::cosh(k * h) / r2;
        if (a > 60.0) break;
        sum += (k == 0 ? 0.5 : 1.0) * std::exp(-a) * std::sin(a);
    }
    return -h * sum;
}

struct KeiTable {
    static constexpr int N = 1001;
    double rn[N], v[N];
    KeiTable()
    {
        char buf[64];
        for (int i = 0; i < N; ++i) {
            const double x = i / 100.0;
            snprintf(buf, sizeof(buf), "%.4f", x);
            rn[i] = (double)strtof(buf, nullptr);
            snprintf(buf, sizeof(buf), "%.4E", kelvin_kei(x));
            v[i] = (double)strtof(buf, nullptr);
        }
    }
    // get_kei_value: linear interpolation, the last value beyond the table
    double at(double r, double L_w) const
    {
        const double q = r / L_w;
        if (q > rn[N - 1]) return v[N - 1];
        int k = (int)(q * 100.0);
        if (k > N - 2) k = N - 2;
        while (k > 0 && q < rn[k]) --k;
        while (k < N - 2 && q >= rn[k + 1]) ++k;
        return v[k] + (q - rn[k]) / (rn[k + 1] - rn[k]) * (v[k + 1] - v[k]);
    }
};

const KeiTable& kei_table()
{
    static const KeiTable t;   // built once, thread-safe
    return t;
}

void fill_rheo_params(const fi_handle* h, RheoParams& P)
{
    const fi_params& p = h->p;
    P.nx = h->nx;
    P.ny = h->ny;
    P.method = p.method;
    P.lithosphere = p.lithosphere;
    P.mantle = p.mantle;
    P.layering = p.layering;
    P.lumping = p.lumping;
    P.nl = p.nl;
    P.visc_scaling_method = p.visc_scaling_method;
    for (int k = 0; k < 8; ++k) { P.zl[k] = p.zl[k]; P.viscosities[k] = p.viscosities[k]; }
    P.dl = p.dl;
    P.E = p.E;
    P.nu = p.nu;
    P.viscosity_scaling = p.viscosity_scaling;
    P.cc = h->cc;
    P.eta_ref = p.eta_ref;
    P.big_he = sp(100e3);   // calc_gaussian_thickness amplitude (src/fastisostasy.f90:250-260)
}

void host_fields(fi_handle* h)
{
    const fi_params& p = h->p;
    const size_t n = h->n;
    h->He.assign(n, p.zl[0]);
    h->D.assign(n, rigidity(p.E, p.zl[0], p.nu));
    h->R.assign(n, 1.0);
    h->eta_eff.assign(n, p.viscosities[p.nl - 1]);
    // kappa, GE and GN cell by cell on the device (host loops as the fallback
    // for a failed launch are not kept: a device error is reported)
    h->kappa.assign(n, 0.0);
    h->GE.assign(n, 0.0);
    h->GN.assign(n, 0.0);
    h->init_rc = init_fields_device(h->nx, h->ny, h->dx, h->dy, PI_LIT, sp(1.e-12), sp(9.81), p.r_earth, p.m_earth,
                                    kRn, kGe, h->kappa.data(), h->GE.data(), h->GN.data(), h->s);
    // He, D and (method 3) eta_eff, R on the device: src/fastisostasy.f90:240-443
    if (!h->init_rc) {
        RheoParams P;
        fill_rheo_params(h, P);
        h->init_rc = rheology_device(P, h->xc.data(), h->yc.data(), h->dx, h->kappa.data(), nullptr, h->He.data(),
                                     h->D.data(), h->eta_eff.data(), h->R.data(), h->s);
    }
    const int nx = h->nx, ny = h->ny;
    const double dx = h->dx;
    // LV-ELRA kernel, src/fastisostasy.f90:216-236: kei filter on the padded
    // domain, GV = -L_w^2 / (2 pi D) kei (dx dy) (src/green_functions.f90:28-41),
    // L_w = (D / (rho_m g))^(1/4) (src/isos_utils.f90:66-73)
    if (p.method == 2) {
        const double Dc = rigidity(p.E, p.zl[0], p.nu);
        h->L_w = std::pow(Dc / (p.rho_uppermantle * p.g), 0.25);
        const KeiTable& kt = kei_table();
        h->GV.assign(n, 0.0);
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double x = h->xc[i], y = h->yc[j];
                const double kei = kt.at(std::sqrt(x * x + y * y), h->L_w);
                h->GV[(size_t)j * nx + i] = -(h->L_w * h->L_w) / (2.0 * PI_LIT * Dc) * kei * (dx * dx);
            }
    }
    // maskactive, src/fastisostasy.f90:185-198; methods 0-2: all active (:444-451)
    h->mact.assign(n, 0);
    if (p.method != 3 || !p.interactive_sealevel) {
        for (auto& m : h->mact) m = 1;
    } else if (p.min_pad > sp(100.e3)) {
        for (int j = h->jcrop1; j <= h->jcrop2; ++j)
            for (int i = h->icrop1; i <= h->icrop2; ++i) h->mact[(size_t)(j - 1) * nx + (i - 1)] = 1;
    }
}

// Upload the derived static fields: D, 1/(2 eta), 1/(kappa R) in the
// spectrum layout, maskactive.
int upload_static(fi_handle* h)
{
    const size_t n = h->n;
    std::vector<double> inv2eta(n);
    for (size_t e = 0; e < n; ++e) inv2eta[e] = 1.0 / (2.0 * h->eta_eff[e]);
    int rc;
    if ((rc = upload_T(h, h->Dt, h->D)) || (rc = upload_T(h, h->inv2eta, inv2eta))) return rc;
    const int nx = h->nx, ny = h->ny, hh = nx / 2, spitch = h->prhs.sp;
    std::vector<double> A((size_t)ny * spitch, 0.0), B((size_t)ny * spitch, 0.0);
    auto m = [&](int k, int l) { return 1.0 / (h->kappa[(size_t)l * nx + k] * h->R[(size_t)l * nx + k]); };
    h->even = 1;
    for (int l = 0; l < ny; ++l)
        for (int k = 0; k <= hh; ++k) {
            A[(size_t)l * spitch + k] = m(k, l);
            B[(size_t)l * spitch + k] = m((nx - k) % nx, l);
        }
    for (int l = 0; l < ny && h->even; ++l)
        for (int k = 0; k < nx; ++k)
            if (m(k, l) != m((nx - k) % nx, l) || m(k, l) != m(k, (ny - l) % ny)) { h->even = 0; break; }
    if ((rc = upload_T(h, h->mA, A)) || (rc = upload_T(h, h->mB, B))) return rc;
    if (h->mAT) {
        std::vector<double> AT((size_t)(hh + 1) * ny), BT((size_t)(hh + 1) * ny);
        for (int k = 0; k <= hh; ++k)
            for (int l = 0; l < ny; ++l) {
                AT[(size_t)k * ny + l] = A[(size_t)l * spitch + k];
                BT[(size_t)k * ny + l] = B[(size_t)l * spitch + k];
            }
        if ((rc = upload_T(h, h->mAT, AT)) || (rc = upload_T(h, h->mBT, BT))) return rc;
    }

    if ((rc = upload(h, (void*)h->d.mactive, h->mact.data(), n))) return rc;
    return FI_OK;
}

// kernel spectrum: zero-padded r2c of a padded-grid kernel (precompute_kernel,
// src/convolutions.f90:93-108), computed in double on the device.
// Autotuner of the single-domain RHS transforms: rows per row-transform
// block and spectrum columns per column-transform block, timed on the
// handle's own buffers (RHS scratch, dead at set-up) and cached per grid
// size and precision for the process.  The step engine has its own shapes.
template <typename T> void tune_rhs_shapes(fi_handle* h)
{
    typedef typename vec2<T>::type C2;
    struct Key {
        int nx, ny, sz;
        bool operator==(const Key& o) const { return nx == o.nx && ny == o.ny && sz == o.sz; }
    };
    static std::mutex mu;
    struct Shape {
        int rb, rt, cb, ct;
    };
    static std::vector<std::pair<Key, Shape>> cache;
    const Key key{h->nx, h->ny, (int)sizeof(T)};
    {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& e : cache)
            if (e.first == key) {
                h->prhs.rb = e.second.rb;
                h->prhs.rt = e.second.rt;
                h->prhs.cb = e.second.cb;
                h->prhs.ct = e.second.ct;
                return;
            }
    }
    int optin = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    Plan2D p = h->prhs;
    auto time_it = [&](auto&& fn) {
        float best = 1e30f;
        for (int r = 0; r < 4; ++r) {
            cudaEventRecord(e0, h->s);
            fn();
            cudaEventRecord(e1, h->s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && ms < best) best = ms;
        }
        return best;
    };
    const double scale = 1.0 / (double)(float)((long long)h->nx * h->ny);
    // rows (columns) per block x threads per block: more threads per
    // block keep more warps resident on long rows, where one block per
    // row of 1024 points at 256 threads left most warp slots empty
    int best_rb = 0, best_cb = 0, best_rt = 0, best_ct = 0;
    float tr = 1e30f, tc = 1e30f;
    for (int rb : {1, 2, 4, 8}) {
        if (2 * (size_t)rb * p.h * sizeof(C2) > (size_t)optin) continue;
        for (int rt : {128, 256, 512, 1024}) {
            if (rt > 128 && rt > rb * p.h / 2) continue;   // at most one element pair per thread
            p.rb = rb;
            p.rt = rt;
            const float t = time_it([&] {
                launch_rows_fwd<T>((const T*)h->f, h->nx, h->nx, h->ny, (C2*)h->S, p, h->s);
                launch_rows_inv<T>((const C2*)h->S, (T*)h->raw[0], p, scale, h->s);
            });
            if (cudaGetLastError() != cudaSuccess) continue;   // a shape the device refuses
            if (t < tr) { tr = t; best_rb = rb; best_rt = rt; }
        }
    }
    for (int cb : {1, 2, 4, 8}) {
        if (2 * (size_t)cb * (p.ny + 1) * sizeof(C2) > (size_t)optin) continue;
        for (int ct : {128, 256, 512, 1024}) {
            if (ct > 128 && ct > cb * p.ny / 2) continue;
            p.cb = cb;
            p.ct = ct;
            const float t = time_it([&] {
                launch_cols_hartley<T>((C2*)h->S, (const T*)h->mA, (const T*)h->mB, h->even, p, h->s);
            });
            if (cudaGetLastError() != cudaSuccess) continue;
            if (t < tc) { tc = t; best_cb = cb; best_ct = ct; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
    h->prhs.rb = best_rb;
    h->prhs.rt = best_rt;
    h->prhs.cb = best_cb;
    h->prhs.ct = best_ct;
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back({key, Shape{best_rb, best_rt, best_cb, best_ct}});
}

int kernel_spectrum(fi_handle* h, const std::vector<double>& ker, int which)
{
    const size_t hs = (size_t)h->pconv.ny * h->pconv.sp;
    double* tmp = nullptr;
    double2* S64 = nullptr;
    int rc;
    // stream-ordered temporaries: no device-wide synchronisation at set-up
    if (cudaMallocAsync((void**)&tmp, h->n * sizeof(double), h->s) != cudaSuccess) return fail(h, FI_E_OOM, "spectrum");
    if (cudaMallocAsync((void**)&S64, hs * sizeof(double2), h->s) != cudaSuccess) {
        cudaFreeAsync(tmp, h->s);
        return fail(h, FI_E_OOM, "spectrum");
    }
    if ((rc = upload(h, tmp, ker.data(), h->n * sizeof(double)))) {
        cudaFreeAsync(tmp, h->s);
        cudaFreeAsync(S64, h->s);
        return rc;
    }
    launch_rows_fwd<double>(tmp, h->nx, h->nx, h->ny, S64, h->pconv, h->s);
    launch_cols_fwd<double>(S64, h->ny, h->pconv, h->s);
    CK(cudaGetLastError());
    if (mixed(h)) {
        if (narrow_spectrum(S64, (float2*)h->KS[which], hs, h->s)) return fail(h, FI_E_CUDA, "spectrum narrowing");
    } else {
        CK(cudaMemcpyAsync(h->KS[which], S64, hs * sizeof(double2), cudaMemcpyDeviceToDevice, h->s));
    }
    cudaFreeAsync(tmp, h->s);
    cudaFreeAsync(S64, h->s);
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

// The convolution transforms (2n-padded grid) by the same search: rows
// (rows per block x threads) over the forward rows and the cropped inverse
// rows, columns (columns per block x threads) over the column pass with the
// kernel multiply.  The shapes go to pconv_run, which only the update's
// convolutions use (the set-up transforms of the kernels keep pconv).
template <typename T> void tune_conv_shapes(fi_handle* h)
{
    typedef typename vec2<T>::type C2;
    struct Key {
        int px, py, sz;
        bool operator==(const Key& o) const { return px == o.px && py == o.py && sz == o.sz; }
    };
    struct Shape {
        int rb, rt, cb, ct;
    };
    static std::mutex mu;
    static std::vector<std::pair<Key, Shape>> cache;
    const Key key{h->Px, h->Py, (int)sizeof(T)};
    h->pconv_run = h->pconv;
    {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& e : cache)
            if (e.first == key) {
                h->pconv_run.rb = e.second.rb;
                h->pconv_run.rt = e.second.rt;
                h->pconv_run.cb = e.second.cb;
                h->pconv_run.ct = e.second.ct;
                return;
            }
    }
    int optin = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    Plan2D p = h->pconv;
    auto time_it = [&](auto&& fn) {
        float best = 1e30f;
        for (int r = 0; r < 4; ++r) {
            cudaEventRecord(e0, h->s);
            fn();
            cudaEventRecord(e1, h->s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && ms < best) best = ms;
        }
        return best;
    };
    const double scale = 1.0 / ((double)h->Px * (double)h->Py);
    int best_rb = 0, best_cb = 0, best_rt = 0, best_ct = 0;
    float tr = 1e30f, tc = 1e30f;
    for (int rb : {1, 2, 4}) {
        if (2 * (size_t)rb * p.h * sizeof(C2) > (size_t)optin) continue;
        for (int rt : {128, 256, 512, 1024}) {
            if (rt > 128 && rt > rb * p.h / 2) continue;   // at most one element pair per thread
            p.rb = rb;
            p.rt = rt;
            const float t = time_it([&] {
                launch_rows_fwd<T>((const T*)h->conv_in, h->nx, h->nx, h->ny, (C2*)h->S2, p, h->s);
                launch_conv_rows_inv<T>((const C2*)h->S2, h->ny + 2, h->we_raw, h->nx, h->ny, h->nx / 2 - 1,
                                        h->corners, 0, 0, 2 * h->nx - 2, p, scale, h->s);
            });
            if (cudaGetLastError() != cudaSuccess) continue;   // a shape the device refuses
            if (t < tr) { tr = t; best_rb = rb; best_rt = rt; }
        }
    }
    p.rb = best_rb;
    p.rt = best_rt;
    for (int cb : {1, 2, 4}) {
        if (2 * (size_t)cb * (p.ny + 1) * sizeof(C2) > (size_t)optin) continue;
        for (int ct : {128, 256, 512, 1024}) {
            if (ct > 128 && ct > cb * p.ny / 2) continue;
            p.cb = cb;
            p.ct = ct;
            const float t = time_it([&] {
                launch_cols_conv<T>((C2*)h->S2, (const C2*)h->KS[0], h->ny, h->out_rows, h->ny + 2, p, h->s);
            });
            if (cudaGetLastError() != cudaSuccess) continue;
            if (t < tc) { tc = t; best_cb = cb; best_ct = ct; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
    h->pconv_run.rb = best_rb;
    h->pconv_run.rt = best_rt;
    h->pconv_run.cb = best_cb;
    h->pconv_run.ct = best_ct;
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back({key, Shape{best_rb, best_rt, best_cb, best_ct}});
}

// ---- device pipelines ------------------------------------------------------
template <typename T> struct TT {
    typedef typename vec2<T>::type C2;
};

// gate: optional device flag; the four kernels return at once when it is 0
// whi/wlo: the state y as a float pair (mixed Tsit5), else null
template <typename T>
void rhs(fi_handle* h, const double* y, const double* wref, T* raw_out, const int* gate = nullptr,
         const float* whi = nullptr, const float* wlo = nullptr)
{
    typedef typename vec2<T>::type C2;
    if (h->p.method != 3) {
        // methods 0-2: (w_eq - y) / tau, w_eq computed once per update
        PROF(h, K_FLEX, relax_rate<T>(raw_out, y, h->weq, h->p.tau, h->n, gate, h->s));
        h->launches += 1;
        return;
    }
    PROF(h, K_FLEX, launch_flexure<T>(y, wref, (const T*)h->q0, h->d.mactive, (const T*)h->Dt, (const T*)h->inv2eta,
                                      (T*)h->f, h->nx, h->ny, h->fc, h->s, gate, whi, wlo));
    PROF(h, K_ROWS_FWD, launch_rows_fwd<T>((const T*)h->f, h->nx, h->nx, h->ny, (C2*)h->S, h->prhs, h->s, gate));
    PROF(h, K_COLS_HARTLEY,
         launch_cols_hartley<T>((C2*)h->S, (const T*)h->mA, (const T*)h->mB, h->even, h->prhs, h->s, gate));
    const double norm = (double)(float)((long long)h->nx * h->ny);   // nx*ny*1. (default real)
    PROF(h, K_ROWS_INV, launch_rows_inv<T>((const C2*)h->S, raw_out, h->prhs, 1.0 / norm, h->s, gate));
    h->launches += 4;
}

// One mixed RK4 stage RHS from the float pair of x (rprev: the previous
// stage's raw RHS, null at the first stage; a: its tableau weight).
void rhs_pair_stage(fi_handle* h, const float* rprev, double a, float* raw_out)
{
    typedef vec2<float>::type C2;
    PROF(h, K_FLEX, launch_flexure_stage(h->xhi, h->xlo, rprev, h->dxw, (const float*)h->q0, h->d.mactive,
                                         (const float*)h->Dt, (const float*)h->inv2eta, (float*)h->f, h->nx, h->ny,
                                         h->fc, h->ctl, a, h->rate_scale, h->s));
    PROF(h, K_ROWS_FWD, launch_rows_fwd<float>((const float*)h->f, h->nx, h->nx, h->ny, (C2*)h->S, h->prhs, h->s));
    PROF(h, K_COLS_HARTLEY,
         launch_cols_hartley<float>((C2*)h->S, (const float*)h->mA, (const float*)h->mB, h->even, h->prhs, h->s));
    const double norm = (double)(float)((long long)h->nx * h->ny);   // nx*ny*1. (default real)
    PROF(h, K_ROWS_INV, launch_rows_inv<float>((const C2*)h->S, raw_out, h->prhs, 1.0 / norm, h->s));
    h->launches += 4;
}

// One RHS of the mixed true-stage Tsit5 at a stage state given as a float
// pair with its dxw (rhs with the column-strip stencil in stage mode).
void rhs_tpair(fi_handle* h, const float* hi, const float* lo, const float* dw, float* raw_out, const int* gate)
{
    typedef vec2<float>::type C2;
    PROF(h, K_FLEX, launch_flexure_stage(hi, lo, nullptr, dw, (const float*)h->q0, h->d.mactive, (const float*)h->Dt,
                                         (const float*)h->inv2eta, (float*)h->f, h->nx, h->ny, h->fc, h->ctl, 0.0,
                                         h->rate_scale, h->s, gate));
    PROF(h, K_ROWS_FWD,
         launch_rows_fwd<float>((const float*)h->f, h->nx, h->nx, h->ny, (C2*)h->S, h->prhs, h->s, gate));
    PROF(h, K_COLS_HARTLEY, launch_cols_hartley<float>((C2*)h->S, (const float*)h->mA, (const float*)h->mB, h->even,
                                                       h->prhs, h->s, gate));
    const double norm = (double)(float)((long long)h->nx * h->ny);   // nx*ny*1. (default real)
    PROF(h, K_ROWS_INV, launch_rows_inv<float>((const C2*)h->S, raw_out, h->prhs, 1.0 / norm, h->s, gate));
    h->launches += 4;
}

template <typename T> void conv(fi_handle* h, int which, double* out_raw, double* corners)
{
    typedef typename vec2<T>::type C2;
    PROF(h, K_CONV_ROWS_FWD,
         launch_rows_fwd<T>((const T*)h->conv_in, h->nx, h->nx, h->ny, (C2*)h->S2, h->pconv_run, h->s));
    PROF(h, K_CONV_COLS, launch_cols_conv<T>((C2*)h->S2, (const C2*)h->KS[which], h->ny, h->out_rows, h->ny + 2,
                                             h->pconv_run, h->s));
    PROF(h, K_CONV_ROWS_INV, launch_conv_rows_inv<T>((const C2*)h->S2, h->ny + 2, out_raw, h->nx, h->ny, h->nx / 2 - 1,
                                                     corners, 0, 0, 2 * h->nx - 2, h->pconv_run,
                                                     1.0 / ((double)h->Px * (double)h->Py), h->s));
    h->launches += 3;
}

// Fixed-step integrators (euler, rk4): the step sequence of one update is
// known on the host from a mirror of the ode clock that repeats the device's
// fmin/add sequence, so an update has a static kernel sequence.
int plan_steps(fi_handle* h, double tf)
{
    const fi_params& p = h->p;
    int n = 0;
    while (h->h_t < tf) {
        double hstep;
        if (p.dt_method == 1) hstep = fmin(h->h_dt, tf - h->h_t);
        else { h->h_dt = fmin(h->h_dt, tf - h->h_t); hstep = h->h_dt; }
        h->h_t = h->h_t + hstep;
        ++n;
    }
    return n;
}

// Enqueue `nsteps` euler/rk4 steps; returns the raw buffer of the last RHS.
template <typename T> T* enqueue_steps(fi_handle* h, int nsteps)
{
    const fi_params& p = h->p;
    const double spy = h->rate_scale;
    T *r0 = (T*)h->raw[0], *r1 = (T*)h->raw[1], *r2 = (T*)h->raw[2], *r3 = (T*)h->raw[3];
    const bool truem = p.stage_mode == 1;
    const double* wref = truem ? h->w_ref : nullptr;
    // mixed true-stage RK4 on a uniform grid: stage states from the float
    // pair of x, as the step engine forms them (no FP64 stage state)
    const bool pairs = sizeof(T) == 4 && truem && p.dt_method == 1 && p.method == 3 && h->dxw != nullptr;
    if (pairs && nsteps > 0) {
        PROF(h, K_STAGE, split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, h->s));
        h->launches += 1;
    }
    T* last = r0;
    for (int st = 0; st < nsteps; ++st) {
        PROF(h, K_CONTROL, step_begin(h->ctl, p.dt_method == 1 ? 1 : 0, h->s));
        if (pairs) {
            rhs_pair_stage(h, nullptr, 0.0, (float*)r0);
            rhs_pair_stage(h, (const float*)r0, 0.5, (float*)r1);
            rhs_pair_stage(h, (const float*)r1, 0.5, (float*)r2);
            rhs_pair_stage(h, (const float*)r2, 1.0, (float*)r3);
            PROF(h, K_RK_FINAL, rk4_final_pair(h->ctl, h->d.x, h->d.w, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw,
                                               (const float*)r0, (const float*)r1, (const float*)r2,
                                               (const float*)r3, h->nx, h->ny, spy, h->s));
            h->launches += 1;
            last = r3;
        } else if (p.dt_method == 1 && truem) {
            rhs<T>(h, h->d.x, wref, r0);
            PROF(h, K_STAGE, rk_stage<T>(h->ctl, h->y, h->d.x, r0, 0.5, h->nx, h->ny, spy, h->s));
            rhs<T>(h, h->y, wref, r1);
            PROF(h, K_STAGE, rk_stage<T>(h->ctl, h->y, h->d.x, r1, 0.5, h->nx, h->ny, spy, h->s));
            rhs<T>(h, h->y, wref, r2);
            PROF(h, K_STAGE, rk_stage<T>(h->ctl, h->y, h->d.x, r2, 1.0, h->nx, h->ny, spy, h->s));
            rhs<T>(h, h->y, wref, r3);
            PROF(h, K_RK_FINAL, rk4_final<T>(h->ctl, h->d.x, h->d.w, r0, r1, r2, r3, h->nx, h->ny, spy, h->s));
            h->launches += 4;
            last = r3;
        } else if (p.dt_method == 1) {
            rhs<T>(h, h->d.w, nullptr, r0);
            PROF(h, K_RK_FINAL, rk4_final<T>(h->ctl, h->d.x, h->d.w, r0, r0, r0, r0, h->nx, h->ny, spy, h->s));
            h->launches += 1;
        } else {
            rhs<T>(h, truem ? h->d.x : h->d.w, wref, r0);
            PROF(h, K_RK_FINAL, euler_final<T>(h->ctl, h->d.x, h->d.w, r0, h->nx, h->ny, spy, h->s));
            h->launches += 1;
        }
        PROF(h, K_CONTROL, step_end(h->ctl, h->s));
        h->launches += 2;
    }
    return last;
}

// All RK4 steps of one update in one cooperative launch (fi_engine.cu).
template <typename T> T* enqueue_engine(fi_handle* h, int nsteps)
{
    if (mixed(h)) {
        PROF(h, K_STAGE, split_hilo(h->d.x, h->xhi, h->xlo, h->n, h->s));
        h->launches += 1;
    }
    EngineArgs g;
    memset(&g, 0, sizeof(g));
    g.p = h->prhs;
    g.fc = h->fc;
    g.x = h->d.x;
    g.w = h->d.w;
    g.xhi = h->xhi;
    g.xlo = h->xlo;
    g.wrefhi = h->wrefhi;
    g.wreflo = h->wreflo;
    g.wref = h->w_ref;
    g.q0 = h->q0;
    g.D = h->Dt;
    g.inv2eta = h->inv2eta;
    g.mA = h->mAT;
    g.mB = h->mBT;
    g.ST = h->ST;
    g.even = h->even;
    g.mask = h->d.mactive;
    for (int i = 0; i < 4; ++i) g.raw[i] = h->raw[i];
    g.S = h->S;
    g.ctl = h->ctl;
    g.nsteps = nsteps;
    g.CB = h->eng_CB;
    g.ra = h->eng_RA;
    g.p2 = h->eng_P2;
    g.spy = h->spy;
    g.norm_scale = 1.0 / (double)(float)((long long)h->nx * h->ny);
    g.norm_scale_f = (float)g.norm_scale;
    g.fcf = flex_coef_f32(h->fc);
    g.trace = h->trace;
    g.bar = h->eng_bar;
    {
        // test only: FI_ENGINE_BARRIER_PHANTOM=1 expects one arrival more than
        // the grid has, so every barrier wait runs out (FI_E_TIMEOUT)
        const char* e = getenv("FI_ENGINE_BARRIER_PHANTOM");
        g.bar_phantom = (e && e[0] == '1') ? 1 : 0;
    }
    cudaError_t le = cudaMemsetAsync(h->eng_bar, 0, sizeof(unsigned), h->s);
    if (le != cudaSuccess && h->launch_err == cudaSuccess) h->launch_err = le;
    PROF(h, K_ENGINE, le = engine_launch<T>(g, h->eng_grid, h->eng_smem, h->s));
    if (le != cudaSuccess && h->launch_err == cudaSuccess) h->launch_err = le;
    h->launches += 1;
    return (T*)h->raw[3];
}

const int kMaxAttempts = 10000000;
const long long kDefaultMaxReject = 1000000;   // rejections per update (fi_set_max_rejections)

// One attempt of Tsitouras 5(4) with true stages (the Dormand-Prince 5(4)
// pair, FSAL), decided on the device: k_0 = f(x) unless an accepted attempt
// left it cached, stage states y_i = x + h sum a_ij k_j with the RHS (mantle
// term at the stage state) evaluated at each, stage 6 = x2, the embedded x1,
// the error norm, the commit and the FSAL copy.
template <typename T> void tsit_true_attempt(fi_handle* h, cudaGraphConditionalHandle loop, int* more_out)
{
    const fi_params& p = h->p;
    DPRaw<T> R;
    for (int i = 0; i < 7; ++i) R.p[i] = (const T*)h->raw[i];
    ts_attempt_begin(h->ctl, kMaxAttempts, h->s);
    if (sizeof(T) == 4 && h->yhi) {
        // mixed form: stage states as float pairs (no FP64 stage state but x2)
        DPRaw<float> Rf;
        for (int i = 0; i < 7; ++i) Rf.p[i] = (const float*)h->raw[i];
        rhs_tpair(h, h->xhi, h->xlo, h->dxw, (float*)h->raw[0], &h->ctl->need_rhs);
        for (int i = 1; i <= 6; ++i) {
            PROF(h, K_STAGE, dp_stage_pair(h->ctl, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->yhi, h->ylo, h->ydw,
                                           i == 6 ? h->d.ts_x2 : nullptr, h->d.x, Rf, i, h->nx, h->ny,
                                           h->rate_scale, h->s));
            rhs_tpair(h, h->yhi, h->ylo, h->ydw, (float*)h->raw[i], &h->ctl->active);
        }
        PROF(h, K_TS, dp_err<T>(h->d, R, p.atol, p.rtol, h->s));
        PROF(h, K_TS, ts_err<T>(h->d, (const T*)h->raw[0], p.q, p.dt_max, h->s));
        PROF(h, K_TS, ts_commit_tpair(h->d, h->xhi, h->xlo, h->dxw, h->yhi, h->ylo, h->ydw, h->s));
        PROF(h, K_TS, fsal_copy<T>(h->ctl, (T*)h->raw[0], (const T*)h->raw[6], h->n, h->s));
        ts_attempt_end(h->ctl, loop, h->s, 1, more_out);
        h->launches += 12;
        return;
    }
    rhs<T>(h, h->d.x, h->w_ref, (T*)h->raw[0], &h->ctl->need_rhs);
    for (int i = 1; i <= 6; ++i) {
        double* y = i == 6 ? h->d.ts_x2 : h->y;
        PROF(h, K_STAGE, dp_stage<T>(h->ctl, y, h->d.x, R, i, h->nx, h->ny, h->rate_scale, h->s));
        rhs<T>(h, y, h->w_ref, (T*)h->raw[i], &h->ctl->active);
    }
    PROF(h, K_TS, dp_err<T>(h->d, R, p.atol, p.rtol, h->s));
    PROF(h, K_TS, ts_err<T>(h->d, (const T*)h->raw[0], p.q, p.dt_max, h->s));
    PROF(h, K_TS, ts_commit<T>(h->d, (const T*)h->raw[0], h->s));
    PROF(h, K_TS, fsal_copy<T>(h->ctl, (T*)h->raw[0], (const T*)h->raw[6], h->n, h->s));
    ts_attempt_end(h->ctl, loop, h->s, 1, more_out);
    h->launches += 12;
}

// Reference-compatible Tsit5: one distinct RHS per state; the host waits
// for each attempt's accept/reject decision.  True stages: the same device
// attempt as in captured graphs, the host only reads the loop condition.
template <typename T> int integrate_tsit(fi_handle* h, double tf, int* have_rhs, T** raw_last)
{
    const fi_params& p = h->p;
    T* r0 = (T*)h->raw[0];
    *have_rhs = 0;
    *raw_last = r0;
    if (p.stage_mode == 1) {
        ts_loop_begin(h->ctl, h->s);
        if (h->yhi) split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, h->s);
        for (long long it = 0;; ++it) {
            tsit_true_attempt<T>(h, 0, h->dmore);
            int more = 0;
            CK(cudaMemcpyAsync(&more, h->dmore, sizeof(int), cudaMemcpyDeviceToHost, h->s));
            CK(cudaStreamSynchronize(h->s));
            if (!more) break;
            if (it > kMaxAttempts) return fail(h, FI_E_STEP, "tsit54: too many attempts");
        }
        *have_rhs = -1;   // recorded on the device
        return FI_OK;
    }
    if (h->d.whi) split_hilo(h->d.w, h->d.whi, h->d.wlo, h->n, h->s);
    Ctl hc;
    CK(cudaMemcpyAsync(&hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    bool need_rhs = true;
    int guard = 0;
    while (hc.t < tf && hc.status == ST_OK) {
        PROF(h, K_CONTROL, step_begin(h->ctl, 2, h->s));
        if (need_rhs) { rhs<T>(h, h->d.w, nullptr, r0, nullptr, h->d.whi, h->d.wlo); *have_rhs = 1; }
        if (sizeof(T) == 4 && h->d.whi) {
            PROF(h, K_TS, ts_fused(h->d, (const float*)r0, p.atol, p.rtol, p.q, p.dt_max, h->s));
            PROF(h, K_TS, ts_commit_pair(h->d, (const float*)r0, h->s));
            h->launches += 3;
        } else {
            PROF(h, K_TS, ts_max<T>(h->d, r0, p.atol, p.rtol, h->s));
            PROF(h, K_TS, ts_err<T>(h->d, r0, p.q, p.dt_max, h->s));
            PROF(h, K_TS, ts_commit<T>(h->d, r0, h->s));
            h->launches += 4;
        }
        CK(cudaMemcpyAsync(&hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
        CK(cudaStreamSynchronize(h->s));
        need_rhs = hc.accepted != 0;
        if (++guard > 10000000) return fail(h, FI_E_STEP, "tsit54: too many attempts");
    }
    return FI_OK;
}

// The same attempts as integrate_tsit, enqueued during stream capture as the
// body of a CUDA graph WHILE node: the accept/reject decisions stay on the
// device.  Only valid while h->s is capturing.
template <typename T> int enqueue_tsit_loop(fi_handle* h)
{
    const fi_params& p = h->p;
    T* r0 = (T*)h->raw[0];
    ts_loop_begin(h->ctl, h->s);
    h->launches += 1;
    if (h->d.whi) {
        split_hilo(h->d.w, h->d.whi, h->d.wlo, h->n, h->s);
        h->launches += 1;
    }
    if (h->yhi) {
        split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, h->s);
        h->launches += 1;
    }
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(h->s, &st, nullptr, &g, &deps, nullptr, &nd));
    if (st != cudaStreamCaptureStatusActive) return fail(h, FI_E_CUDA, "tsit54 loop: stream is not capturing");
    cudaGraphConditionalHandle loop;
    CK(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CK(cudaStreamUpdateCaptureDependencies(h->s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    CK(cudaStreamBeginCaptureToGraph(h->s_body, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaStream_t s0 = h->s;
    h->s = h->s_body;
    if (p.stage_mode == 1) {
        tsit_true_attempt<T>(h, loop, nullptr);
    } else {
        ts_attempt_begin(h->ctl, kMaxAttempts, h->s);
        rhs<T>(h, h->d.w, nullptr, r0, &h->ctl->need_rhs, h->d.whi, h->d.wlo);
        if (sizeof(T) == 4 && h->d.whi) {
            ts_fused(h->d, (const float*)r0, p.atol, p.rtol, p.q, p.dt_max, h->s);
            ts_commit_pair(h->d, (const float*)r0, h->s);
            h->launches -= 1;
        } else {
            ts_max<T>(h->d, r0, p.atol, p.rtol, h->s);
            ts_err<T>(h->d, r0, p.q, p.dt_max, h->s);
            ts_commit<T>(h->d, r0, h->s);
        }
        ts_attempt_end(h->ctl, loop, h->s);
        h->launches += 5;
    }
    h->s = s0;
    cudaGraph_t body_out = nullptr;
    CK(cudaStreamEndCapture(h->s_body, &body_out));
    return FI_OK;
}

// Kernels of isos_update before the integrator (src/fastisostasy.f90:750-833).
template <typename T> void enqueue_pre(fi_handle* h, const double* dH, bool diag, bool run_integrator)
{
    const fi_params& p = h->p;
    PROF(h, K_UPD_BEGIN, upd_begin(h->d, dH, h->s));
    T* cin = (T*)h->conv_in;
    PROF(h, K_UPD_MASKS, upd_masks<T>(h->d, (diag && p.include_elastic) ? cin : (T*)nullptr, h->s));
    int we_mode = 0, dz_mode = 0;
    if (diag) {
        if (p.include_elastic) { conv<T>(h, 0, h->we_raw, h->corners); we_mode = 1; }
        else we_mode = 2;
    }
    PROF(h, K_UPD_LITHO,
         upd_litho<T>(h->d, h->we_raw, h->corners, we_mode, (diag && p.heterogeneous_ssh) ? cin : (T*)nullptr, h->s));
    if (diag) {
        if (p.heterogeneous_ssh) { conv<T>(h, 1, h->dz_raw, h->corners + 4); dz_mode = 1; }
        else dz_mode = 2;
    }
    PROF(h, K_UPD_LOAD, upd_load<T>(h->d, h->dz_raw, h->corners + 4, dz_mode, (T*)h->q0, p.stage_mode,
                                    run_integrator ? 1 : 0, h->s));
    h->launches += 4;
    if (p.method == 0 || p.method == 1) {
        // LLRA equilibrium -canom_load / rho_m (zero for method 0)
        weq_local(h->weq, h->d.c_load, p.rho_uppermantle, p.method == 0 ? 1 : 0, h->n, h->s);
        h->launches += 1;
    } else if (p.method == 2) {
        // LV-ELRA: (-canom_load g K^2) convolved with GV, corner BCs
        elra_load<T>((T*)h->conv_in, h->d.c_load, h->d.K2, p.g, h->n, h->s);
        conv<T>(h, 2, h->weq_raw, h->corners + 8);
        weq_elra(h->weq, h->weq_raw, h->corners + 8, h->nx, h->ny, h->s);
        h->launches += 2;
    }
}

// The tail: corner BC of w, canom_mantle, z_bed, dwdt, checks (:856-869).
template <typename T> void enqueue_post(fi_handle* h, T* raw_last, int have_rhs)
{
    PROF(h, K_UPD_END, upd_end<T>(h->d, raw_last, have_rhs, h->s));
    h->launches += 2;
}

// The body of isos_update on the device (src/fastisostasy.f90:731-872).
// Euler/RK4 updates are captured once per (diagnostics, step count) into a
// CUDA graph and replayed; the per-update scalars were written into the
// control block by enqueue_args just before.
template <typename T> int update_T(fi_handle* h, const double* dH, double time, bool run_integrator)
{
    const fi_params& p = h->p;
    bool diag = false;
    if (time - h->time_diag >= sp(1e-3)) {   // :782-787
        diag = true;
        h->time_diag = h->time_diag + p.dt_diagnostics;
    }
    h->time_prog = time;
    const bool tsit = p.dt_method == 2 && run_integrator;
    const int nsteps = (run_integrator && !tsit) ? plan_steps(h, time) : 0;
    const long long key = ((long long)nsteps << 4) | ((long long)tsit << 3) | ((long long)(dH == h->dH) << 2) |
                          ((diag ? 1 : 0) << 1) | (run_integrator ? 1 : 0);
    // eager: Tsit5 attempts are decided on the host (one wait per attempt)
    auto enqueue = [&]() -> int {
        enqueue_pre<T>(h, dH, diag, run_integrator);
        if (tsit) {
            int have_rhs = 0;
            T* raw_last = nullptr;
            const int rc = integrate_tsit<T>(h, time, &have_rhs, &raw_last);
            if (rc) return rc;
            enqueue_post<T>(h, raw_last, have_rhs);
            return FI_OK;
        }
        T* raw_last = (h->engine_ok && nsteps > 0) ? enqueue_engine<T>(h, nsteps) : enqueue_steps<T>(h, nsteps);
        enqueue_post<T>(h, raw_last, nsteps > 0 ? 1 : 0);
        return FI_OK;
    };
    // captured: Tsit5 attempts loop on the device (graph WHILE node)
    auto enqueue_captured = [&]() -> int {
        if (!tsit) return enqueue();
        enqueue_pre<T>(h, dH, diag, true);
        const int rc = enqueue_tsit_loop<T>(h);
        if (rc) return rc;
        enqueue_post<T>(h, (T*)h->raw[0], -1);
        return FI_OK;
    };
    // the status of the engine's cooperative launch, which the enqueue path
    // records instead of returning: a refused launch fails this update, also
    // inside a stream capture, instead of leaving a step sequence that did
    // nothing
    auto launch_status = [&]() -> int {
        const cudaError_t le = h->launch_err;
        h->launch_err = cudaSuccess;
        if (le != cudaSuccess) return fail(h, FI_E_CUDA, "engine launch: %s", cudaGetErrorString(le));
        return FI_OK;
    };
    if (!h->use_graphs || h->prof_on || (tsit && !h->tsit_graph_ok)) {
        const int rc = enqueue();
        if (rc) return rc;
        if (const int lrc = launch_status()) return lrc;
        CK(cudaGetLastError());
        return FI_OK;
    }
    for (auto& g : h->graphs)
        if (g.key == key) {
            CK(cudaGraphLaunch(g.exec, h->s));
            h->launches += g.nkernels;
            return FI_OK;
        }
    bool seen = false;
    for (long long k : h->graph_seen) seen |= (k == key);
    if (!seen) {
        // first occurrence runs eagerly (also sets kernel attributes)
        h->graph_seen.push_back(key);
        const int rc = enqueue();
        if (rc) return rc;
        if (const int lrc = launch_status()) return lrc;
        CK(cudaGetLastError());
        return FI_OK;
    }
    const long long l0 = h->launches;
    CK(cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_captured();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->s, &graph);
    if (e == cudaSuccess && h->launch_err != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return launch_status();
    }
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        h->launch_err = cudaSuccess;
        if (tsit && rc != FI_E_CONFIG && !h->require_tsit_graph) {
            // no conditional graph nodes here: keep deciding Tsit5 attempts on the host
            h->tsit_graph_ok = false;
            h->err.clear();
            h->launches = l0;
            const int rc2 = enqueue();
            if (rc2) return rc2;
            if (const int lrc = launch_status()) return lrc;
            CK(cudaGetLastError());
            return FI_OK;
        }
        if (rc) return rc;
        return fail(h, FI_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
    }
    fi_handle::GraphEntry ge;
    ge.key = key;
    ge.nkernels = h->launches - l0;
    e = cudaGraphInstantiate(&ge.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(h, FI_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    h->graphs.push_back(ge);
    CK(cudaGraphLaunch(ge.exec, h->s));
    return FI_OK;
}

int update_any(fi_handle* h, const double* dH, double time, bool run_integrator)
{
    return mixed(h) ? update_T<float>(h, dH, time, run_integrator) : update_T<double>(h, dH, time, run_integrator);
}

// Per-update scalars (target time, barystatic sea level, ocean area) go to
// the control block through a kernel argument: no host wait.
void enqueue_args(fi_handle* h, double tf, const fi_bsl* b, bool write_bsl)
{
    set_args(h->ctl, tf, b->bsl_now, b->A_ocean_now, b->method, write_bsl ? 1 : 0, h->s);
    h->launches += 1;
}

int decode_status(fi_handle* h, const Ctl* hc)
{
    switch (hc->status) {
    case ST_OK: return FI_OK;
    case ST_NAN: return fail(h, FI_E_NAN, "isos_update: NaNs detected");
    case ST_LARGE: return fail(h, FI_E_LARGE, "large_check: large values detected (|w| %.3g, |we| %.3g, |dz_ss| %.3g)",
                                hc->red[0], hc->red[1], hc->red[2]);
    case ST_STEP: return fail(h, FI_E_STEP, "adaptive step rejected too often");
    case ST_TIMEOUT: return fail(h, FI_E_TIMEOUT, "step engine: a grid barrier wait expired");
    default: return fail(h, FI_E_CUDA, "unknown device status %d", hc->status);
    }
}

int read_status(fi_handle* h, Ctl* hc)
{
    CK(cudaMemcpyAsync(hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return decode_status(h, hc);
}

}  // namespace

// ============================================================================
extern "C" {

int fi_version(void) { return 1; }

void* fi_stream(fi_handle* h) { return h ? (void*)h->s : nullptr; }

int fi_set_stream(fi_handle* h, void* stream)
{
    if (!h) return FI_E_ARG;
    if (h->s_out) CK(cudaStreamSynchronize(h->s_out));
    CK(cudaStreamSynchronize(h->s));
    if (!h->s_own) h->s_own = h->s;   // the stream the handle created, destroyed with it
    h->s = stream ? (cudaStream_t)stream : h->s_own;
    return FI_OK;
}

long long fi_launch_count(const fi_handle* h) { return h ? h->launches : -1; }

int fi_engine_trace(fi_handle* h, unsigned long long* out, int n)
{
    if (!h) return FI_E_ARG;
    if (!h->trace) {
        int rc;
        if ((rc = dalloc(h, &h->trace, 256 * sizeof(unsigned long long)))) return rc;
        CK(cudaMemsetAsync(h->trace, 0, 256 * sizeof(unsigned long long), h->s));
        CK(cudaStreamSynchronize(h->s));
        return FI_OK;
    }
    if (!out) return FI_OK;
    CK(cudaStreamSynchronize(h->s));
    CK(cudaMemcpy(out, h->trace, (n < 256 ? n : 256) * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    return FI_OK;
}

int fi_profile(fi_handle* h, int enable)
{
    if (!h) return FI_E_ARG;
    prof_collect(h);
    if (enable < 0) {
        for (int i = 0; i < 32; ++i) { h->prof_ms[i] = 0.0; h->prof_cnt[i] = 0; }
    } else {
        h->prof_on = enable != 0;
    }
    return FI_OK;
}

int fi_profile_read(fi_handle* h, double* ms, long long* counts, int n)
{
    if (!h || !ms || !counts) return FI_E_ARG;
    prof_collect(h);
    for (int i = 0; i < n && i < 32; ++i) { ms[i] = h->prof_ms[i]; counts[i] = h->prof_cnt[i]; }
    return FI_OK;
}

const char* fi_last_error(const fi_handle* h) { return h ? h->err.c_str() : "null handle"; }

namespace {
// init_domain_size (src/isos_utils.f90:285-354): padded size and 1-based crop
// window {nx, ny, icrop1, icrop2, jcrop1, jcrop2}; allocates nothing.
int padded_domain(const fi_params& p, int nx_ice, int ny_ice, double dx, double dy, int* pd)
{
    if (p.method < 0 || p.method > 3 || nx_ice < 3 || ny_ice < 3 || p.nl < 1 || p.nl > 8) return FI_E_CONFIG;
    if (dx != dy || p.min_pad < 0.0) return FI_E_CONFIG;   // src/isos_utils.f90:292-300
    int nx_tmp = nx_ice, ny_tmp = ny_ice, npx, npy, nx, ny;
    int icrop1 = 1, jcrop1 = 1;
    if (nx_ice % 2) { icrop1++; nx_tmp++; }
    if (ny_ice % 2) { jcrop1++; ny_tmp++; }
    if (p.nx_target > 0 && p.ny_target > 0) {
        if (p.nx_target < nx_tmp || p.ny_target < ny_tmp || (p.nx_target - nx_tmp) % 2 || (p.ny_target - ny_tmp) % 2)
            return FI_E_CONFIG;
        npx = (p.nx_target - nx_tmp) / 2;
        npy = (p.ny_target - ny_tmp) / 2;
        nx = p.nx_target;
        ny = p.ny_target;
    } else {
        const int npxy = (int)std::lround(p.min_pad / dx);
        npx = npy = npxy;
        if (nx_tmp < ny_tmp) npx += (ny_tmp - nx_tmp) / 2;
        else if (nx_tmp > ny_tmp) npy += (nx_tmp - ny_tmp) / 2;
        nx = nx_tmp + 2 * npx;
        ny = ny_tmp + 2 * npy;
    }
    if (nx > 2048 || ny > 2048) return FI_E_CONFIG;   // column FFT of 2n must fit in shared memory
    if (p.method == 2 && nx != ny) return FI_E_CONFIG;  // calc_kei_filter_2D needs a square domain
    pd[0] = nx;
    pd[1] = ny;
    pd[2] = icrop1 + npx;
    pd[3] = nx - npx;
    pd[4] = jcrop1 + npy;
    pd[5] = ny - npy;
    return FI_OK;
}
}  // namespace

int fi_padded_dims(const fi_params* p, int nx_ice, int ny_ice, double dx, double dy, int32_t* out6)
{
    if (!p || !out6) return FI_E_ARG;
    int pd[6];
    if (int rc = padded_domain(*p, nx_ice, ny_ice, dx, dy, pd)) return rc;
    for (int i = 0; i < 6; ++i) out6[i] = pd[i];
    return FI_OK;
}

int fi_create(const fi_params* pin, int nx_ice, int ny_ice, double dx, double dy, const double* K_or_null,
              fi_handle** out)
{
    ApiRange nr("fi_create");
    if (!pin || !out) return FI_E_ARG;
    *out = nullptr;
    const fi_params& p = *pin;
    int pd[6];
    if (int rc = padded_domain(p, nx_ice, ny_ice, dx, dy, pd)) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return FI_E_CUDA;
    fi_handle* h = new fi_handle();
    h->p = p;
    h->dx = dx;
    h->dy = dy;
    h->nx_ice = nx_ice;
    h->ny_ice = ny_ice;
    h->nx = pd[0];
    h->ny = pd[1];
    h->icrop1 = pd[2];
    h->icrop2 = pd[3];
    h->jcrop1 = pd[4];
    h->jcrop2 = pd[5];
    h->n = (size_t)h->nx * h->ny;
    h->spy = (double)(3600.0f * 24.0f * 365.25f);   // src/fastisostasy.f90:158
    h->rate_scale = p.method == 3 ? h->spy : 1.0;
    h->cc = p.correct_compression ? 1.5 / (1 + p.nu) : 1.0;
    h->Vden = p.rho_ice / p.rho_water - p.rho_ice / p.rho_seawater;
    h->time_diag = sp(1e10);
    h->time_prog = sp(1e10);
    h->xc.resize(h->nx);
    h->yc.resize(h->ny);
    for (int i = 1; i <= h->nx; ++i) h->xc[i - 1] = (i - h->nx / 2 - 1) * dx;   // init_dims
    for (int j = 1; j <= h->ny; ++j) h->yc[j - 1] = (j - h->ny / 2 - 1) * dy;
    h->K.assign(h->n, 1.0);
    if (K_or_null) {
        for (size_t e = 0; e < h->n; ++e) { h->K[e] = K_or_null[e]; if (h->K[e] != 1.0) h->uniform = 0; }
    }
    if (cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess) { delete h; return FI_E_CUDA; }
    if (cudaStreamCreateWithFlags(&h->s_body, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(h->s);
        delete h;
        return FI_E_CUDA;
    }
    if (const char* ev = getenv("FI_NO_GRAPHS")) h->use_graphs = !(ev[0] == '1');
    if (const char* ev = getenv("FI_REQUIRE_TSIT_GRAPH")) h->require_tsit_graph = (ev[0] == '1');
    *out = h;
    host_fields(h);
    if (h->init_rc) return fail(h, FI_E_CUDA, "device init of kappa and the Green's functions failed");

    // ---- device buffers
    const size_t n = h->n;
    const size_t nT = n * tsz(h);
    const size_t nice_ = (size_t)nx_ice * ny_ice;
    Dom& d = h->d;
    memset(&d, 0, sizeof(d));
    d.nx = h->nx;
    d.ny = h->ny;
    d.n = n;
    d.i0 = h->icrop1 - 1;
    d.j0 = h->jcrop1 - 1;
    d.nxi = h->icrop2 - h->icrop1 + 1;
    d.nyi = h->jcrop2 - h->jcrop1 + 1;
    d.interactive = p.interactive_sealevel;
    d.rho_ice = p.rho_ice;
    d.rho_w = p.rho_water;
    d.rho_m = p.rho_uppermantle;
    d.rho_l = p.rho_litho;
    d.g = p.g;
    d.Vden = h->Vden;
    d.spy = h->rate_scale;
    d.rho_sw_over_ice = p.rho_seawater / p.rho_ice;
    d.rho_ice_over_sw = p.rho_ice / p.rho_seawater;
    int rc = 0;
    double *A, *K2;
    uint8_t* mact;
#define AL(ptr, bytes) if ((rc = dalloc(h, &(ptr), (bytes)))) return rc
    AL(A, n * 8); AL(K2, n * 8); AL(mact, n);
    d.A = A; d.K2 = K2; d.mactive = mact;
    AL(h->z_bed_ref, n * 8); AL(h->Hice_ref, n * 8); AL(h->Haf_ref, n * 8); AL(h->z_ss_ref, n * 8);
    AL(h->we_ref, n * 8); AL(h->w_ref, n * 8); AL(h->dz_ss_ref, n * 8);
    AL(h->mo_ref, n); AL(h->mg_ref, n); AL(h->mc_ref, n);
    d.z_bed_ref = h->z_bed_ref; d.Hice_ref = h->Hice_ref; d.Haf_ref = h->Haf_ref; d.z_ss_ref = h->z_ss_ref;
    d.we_ref = h->we_ref; d.w_ref = h->w_ref;
    AL(d.z_bed, n * 8); AL(d.w, n * 8); AL(d.wout, n * 8); AL(d.we, n * 8); AL(d.Haf, n * 8); AL(d.Hice, n * 8);
    AL(d.z_ss, n * 8); AL(d.dz_ss, n * 8); AL(d.dwdt, n * 8); AL(d.x, n * 8);
    AL(d.c_ice, n * 8); AL(d.c_sw, n * 8); AL(d.c_litho, n * 8); AL(d.c_mantle, n * 8); AL(d.c_load, n * 8);
    AL(d.c_full, n * 8); AL(d.mass, n * 8);
    AL(d.m_ocean, n); AL(d.m_grounded, n); AL(d.m_cont, n);
    AL(h->ctl, sizeof(Ctl));
    d.ctl = h->ctl;
    AL(d.partials, (size_t)reduce_blocks(n) * 4 * sizeof(double));
    if (p.dt_method == 2) {
        AL(d.ts_x2, n * sizeof(double));
        AL(d.ts_dx, n * sizeof(double));
        if (mixed(h) && h->uniform && p.stage_mode == 0) {
            AL(d.whi, n * sizeof(float));
            AL(d.wlo, n * sizeof(float));
        }
    }
    AL(h->y, n * 8);
    AL(h->q0, nT); AL(h->Dt, nT); AL(h->inv2eta, nT); AL(h->f, nT);
    for (int i = 0; i < 4; ++i) AL(h->raw[i], nT);
    if (p.dt_method == 2 && p.stage_mode == 1) {
        for (int i = 4; i < 7; ++i) AL(h->raw[i], nT);
        AL(h->dmore, sizeof(int));
    }
    // RHS transform plan
    if ((rc = make_plan(h, h->nx, h->ny, h->prhs))) return rc;
    const size_t c2 = 2 * tsz(h);
    AL(h->S, (size_t)h->ny * h->prhs.sp * c2);
    AL(h->mA, (size_t)h->ny * h->prhs.sp * tsz(h));
    AL(h->mB, (size_t)h->ny * h->prhs.sp * tsz(h));
    // convolution plan: any even size >= 2n-1 gives the reference's linear convolution
    h->Px = nice_even_at_least(2 * h->nx - 1);
    h->Py = nice_even_at_least(2 * h->ny - 1);
    if (h->Px == 2 * h->nx - 2 + 2 && false) {}
    if ((rc = make_plan(h, h->Px, h->Py, h->pconv))) return rc;
    AL(h->S2, (size_t)h->Py * h->pconv.sp * c2);
    AL(h->KS[0], (size_t)h->Py * h->pconv.sp * c2);
    AL(h->KS[1], (size_t)h->Py * h->pconv.sp * c2);
    if (p.method == 2) { AL(h->KS[2], (size_t)h->Py * h->pconv.sp * c2); }
    AL(h->conv_in, nT);
    AL(h->we_raw, n * 8); AL(h->dz_raw, n * 8); AL(h->corners, 12 * sizeof(double));
    if (p.method != 3) {
        AL(h->weq, n * 8);
        if (p.method == 2) { AL(h->weq_raw, n * 8); }
    }
    AL(h->out_rows, (h->ny + 2) * sizeof(int));
    {
        std::vector<int> rows(h->ny + 2);
        for (int j = 0; j < h->ny; ++j) rows[j] = h->ny / 2 - 1 + j;   // crop, src/convolutions.f90:29-55
        rows[h->ny] = 0;
        rows[h->ny + 1] = 2 * h->ny - 2;
        if ((rc = upload(h, h->out_rows, rows.data(), rows.size() * sizeof(int)))) return rc;
    }
    AL(h->dH, nice_ * 8);
    const int nout = 11;
    AL(h->dpack, nice_ * nout * 8);
    h->hpin_elems = nice_ * nout;
    if (cudaMallocHost((void**)&h->hpin, h->hpin_elems * sizeof(double)) != cudaSuccess)
        return fail(h, FI_E_OOM, "cudaMallocHost failed");
    AL(h->gsrc, 8 * sizeof(double*));
    AL(h->gmsrc, 3 * sizeof(uint8_t*));
    {
        const double* src[8] = {d.z_bed, d.z_ss, d.dz_ss, d.w, d.we, d.dwdt, d.c_full, d.Hice};
        const uint8_t* msrc[3] = {d.m_ocean, d.m_grounded, d.m_cont};
        if ((rc = upload(h, (void*)h->gsrc, src, sizeof(src))) || (rc = upload(h, (void*)h->gmsrc, msrc, sizeof(msrc))))
            return rc;
    }
    // static fields
    {
        std::vector<double> Av(n), K2v(n), dxm(n), dym(n);
        for (size_t e = 0; e < n; ++e) {
            dxm[e] = dx * h->K[e];   // src/fastisostasy.f90:152-155
            dym[e] = dy * h->K[e];
            Av[e] = dxm[e] * dym[e];
            K2v[e] = h->K[e] * h->K[e];
        }
        if ((rc = upload(h, A, Av.data(), n * 8)) || (rc = upload(h, K2, K2v.data(), n * 8))) return rc;
        memset(&h->fc, 0, sizeof(h->fc));
        h->fc.nu = p.nu;
        h->fc.one_minus_nu = 1.0 - p.nu;
        h->fc.coef_mantle = -p.g * p.rho_uppermantle;
        h->fc.inv_dx = 1.0 / dx;
        h->fc.inv_2dx = 1.0 / (2 * dx);
        h->fc.inv_dx2 = 1.0 / (dx * dx);
        h->fc.inv_dy = 1.0 / dy;
        h->fc.inv_2dy = 1.0 / (2 * dy);
        h->fc.inv_dy2 = 1.0 / (dy * dy);
        if (!h->uniform) {
            AL(h->dxm, n * 8);
            AL(h->dym, n * 8);
            if ((rc = upload(h, h->dxm, dxm.data(), n * 8)) || (rc = upload(h, h->dym, dym.data(), n * 8))) return rc;
            h->fc.dxm = h->dxm;
            h->fc.dym = h->dym;
        }
    }
#undef AL
    // cooperative step engine for true-stage RK4 on uniform grids; where it
    // does not fit (or FI_NO_ENGINE=1) the mixed form's kernel sequence forms
    // the same stage states from the float pairs
    {
        const char* ev = getenv("FI_NO_ENGINE");
        const bool rk4_true = p.method == 3 && p.stage_mode == 1 && p.dt_method == 1 && h->uniform;
        const bool tsit_true = p.method == 3 && p.stage_mode == 1 && p.dt_method == 2 && h->uniform;
        const bool want = rk4_true && !(ev && ev[0] == '1');
#define AL2(ptr, bytes) if ((rc = dalloc(h, &(ptr), (bytes)))) return rc
        if (want) {
            int ok = mixed(h) ? engine_config<float>(h->prhs, &h->eng_grid, &h->eng_CB, &h->eng_smem, &h->eng_RA,
                                                  &h->eng_P2)
                              : engine_config<double>(h->prhs, &h->eng_grid, &h->eng_CB, &h->eng_smem, &h->eng_RA,
                                                      &h->eng_P2);
            h->engine_ok = ok != 0;
            cudaGetLastError();
            if (h->engine_ok) {
                const size_t nk = (size_t)(h->prhs.h + 1) * h->ny;
                AL2(h->ST, nk * c2); AL2(h->mAT, nk * tsz(h)); AL2(h->mBT, nk * tsz(h));
                AL2(h->eng_bar, sizeof(unsigned));
            }
        }
        if ((rk4_true || tsit_true) && mixed(h)) {
            // the float pairs of x and w_ref (the stage states of every path)
            AL2(h->xhi, n * 4); AL2(h->xlo, n * 4); AL2(h->wrefhi, n * 4); AL2(h->wreflo, n * 4);
            if (!h->engine_ok) AL2(h->dxw, n * 4);
        }
        if (tsit_true && mixed(h)) { AL2(h->yhi, n * 4); AL2(h->ylo, n * 4); AL2(h->ydw, n * 4); }
#undef AL2
    }
    if ((rc = upload_static(h))) return rc;
    h->pconv_run = h->pconv;
    if ((p.include_elastic || p.heterogeneous_ssh) && !(getenv("FI_NO_TUNE") && getenv("FI_NO_TUNE")[0] == '1')) {
        if (mixed(h)) tune_conv_shapes<float>(h);
        else tune_conv_shapes<double>(h);
    }
    if (p.method == 3 && !h->engine_ok && !(getenv("FI_NO_TUNE") && getenv("FI_NO_TUNE")[0] == '1')) {
        if (mixed(h)) tune_rhs_shapes<float>(h);
        else tune_rhs_shapes<double>(h);
        CK(cudaGetLastError());
    }
    if ((rc = kernel_spectrum(h, h->GE, 0)) || (rc = kernel_spectrum(h, h->GN, 1))) return rc;
    if (p.method == 2 && (rc = kernel_spectrum(h, h->GV, 2))) return rc;
    // zero_init_state (src/fastisostasy.f90:505-548): z_bed background 1e6
    {
        std::vector<double> bg(n, 1e6);
        if ((rc = upload(h, d.z_bed, bg.data(), n * 8)) || (rc = upload(h, h->z_bed_ref, bg.data(), n * 8))) return rc;
        Ctl c0;
        memset(&c0, 0, sizeof(c0));
        // methods 0-2 produce the rate itself: no corner mean, no sec/yr
        c0.plain = p.method != 3 ? 1 : 0;
        c0.dt_min = p.dt_min;
        c0.max_reject = kDefaultMaxReject;
        if ((rc = upload(h, h->ctl, &c0, sizeof(c0)))) return rc;
    }
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

int fi_destroy(fi_handle* h)
{
    ApiRange nr("fi_destroy");
    if (!h) return FI_OK;
    // per-run metrics sink: one JSON line per handle, appended to the file
    // FI_METRICS_FILE names
    if (const char* path = getenv("FI_METRICS_FILE")) {
        if (path[0]) {
            char line[1024];
            if (fi_metrics_json(h, line, sizeof(line)) == FI_OK) {
                static std::mutex mu;
                std::lock_guard<std::mutex> lk(mu);
                if (FILE* f = fopen(path, "a")) {
                    fprintf(f, "%s\n", line);
                    fclose(f);
                }
            }
        }
    }
    if (h->s_out) cudaStreamSynchronize(h->s_out);
    if (h->s) {
        for (void* p : h->allocs) cudaFreeAsync(p, h->s);
        cudaStreamSynchronize(h->s);
    } else {
        for (void* p : h->allocs) cudaFree(p);
    }
    if (h->hpin) cudaFreeHost(h->hpin);
    if (h->hctl) cudaFreeHost(h->hctl);
    for (cudaEvent_t e : h->ev_field)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->prof_ev) cudaEventDestroy(e);
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
    if (h->s_out) {
        cudaStreamSynchronize(h->s_out);
        cudaStreamDestroy(h->s_out);
    }
    if (h->ev_snap) cudaEventDestroy(h->ev_snap);
    if (h->ev_out) cudaEventDestroy(h->ev_out);
    if (h->s_own) cudaStreamDestroy(h->s_own);   // h->s is the caller's then
    else if (h->s) cudaStreamDestroy(h->s);
    if (h->s_body) cudaStreamDestroy(h->s_body);
    delete h;
    return FI_OK;
}

int64_t fi_output_bytes(const fi_handle* h)
{
    if (!h) return -1;
    return (int64_t)h->nx_ice * h->ny_ice * 11 * 8;
}

int fi_output_async(fi_handle* h, double* dst)
{
    if (!h || !dst) return FI_E_ARG;
    if (!h->state_ready) return fail(h, FI_E_STATE, "fi_output_async before fi_init_state");
    const size_t ni = (size_t)h->nx_ice * h->ny_ice;
    if (!h->s_out) {
        int rc;
        if ((rc = dalloc(h, &h->dsnap, ni * 11 * 8))) return rc;
        CK(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_snap, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming));
    }
    // the previous snapshot's copy must have left the staging buffer
    if (h->out_pending) CK(cudaStreamWaitEvent(h->s, h->ev_out, 0));
    gather(h->gsrc, h->gmsrc, 8, 3, h->d, h->dsnap, h->s);
    CK(cudaGetLastError());
    h->launches += 1;
    CK(cudaEventRecord(h->ev_snap, h->s));
    CK(cudaStreamWaitEvent(h->s_out, h->ev_snap, 0));
    CK(cudaMemcpyAsync(dst, h->dsnap, ni * 11 * 8, cudaMemcpyDeviceToHost, h->s_out));
    CK(cudaEventRecord(h->ev_out, h->s_out));
    h->out_pending = true;
    return FI_OK;
}

int fi_output_wait(fi_handle* h)
{
    if (!h) return FI_E_ARG;
    if (!h->out_pending) return FI_OK;
    CK(cudaEventSynchronize(h->ev_out));
    h->out_pending = false;
    return FI_OK;
}

int fi_dims(const fi_handle* h, int32_t* o)
{
    if (!h || !o) return FI_E_ARG;
    o[0] = h->nx; o[1] = h->ny; o[2] = h->icrop1; o[3] = h->icrop2; o[4] = h->jcrop1; o[5] = h->jcrop2;
    o[6] = h->nx_ice; o[7] = h->ny_ice;
    return FI_OK;
}

int fi_set_fields(fi_handle* h, const double* D_lith, const double* eta_eff, const double* R, const uint8_t* mask)
{
    if (!h) return FI_E_ARG;
    const size_t n = h->n;
    if (D_lith) h->D.assign(D_lith, D_lith + n);
    if (eta_eff) h->eta_eff.assign(eta_eff, eta_eff + n);
    if (R) h->R.assign(R, R + n);
    if (mask) h->mact.assign(mask, mask + n);
    return upload_static(h);
}

int fi_set_rheology(fi_handle* h, const fi_rheology* r)
{
    if (!h || !r) return FI_E_ARG;
    if (h->p.method != 3) return fail(h, FI_E_ARG, "fi_set_rheology: LV-ELVA (method 3) only");
    if (!r->litho_thickness && !r->log10_viscosity) return FI_OK;
    if (r->nx < 2 || r->ny < 2 || !r->xc || !r->yc || (r->log10_viscosity && (r->nz < 1 || !r->zc)))
        return fail(h, FI_E_ARG, "fi_set_rheology: file grid");
    RheoParams P;
    fill_rheo_params(h, P);
    RheoFile F;
    F.nxr = r->nx;
    F.nyr = r->ny;
    F.nzr = r->nz;
    F.xr = r->xc;
    F.yr = r->yc;
    F.zr = r->zc;
    F.thick = r->litho_thickness;
    F.thick_scale = r->litho_thickness_scaling;
    F.log10_eta = r->log10_viscosity;
    F.stddev = r->stddev_log10_viscosity;
    F.use_stddev = r->stddev_scaling;
    F.smooth_radius = r->rheo_smoothing_radius;
    std::vector<double> He(h->He), D(h->D), eta(h->eta_eff), R(h->R);
    // without a thickness in the file, He (and so the layer boundaries)
    // follows the lithosphere code as at creation
    const int rc = rheology_device(P, h->xc.data(), h->yc.data(), h->dx, h->kappa.data(), &F, He.data(), D.data(),
                                   eta.data(), R.data(), h->s);
    if (rc == 2) return fail(h, FI_E_ARG, "fi_set_rheology: smoothing window wider than the grid");
    if (rc) return fail(h, FI_E_CUDA, "fi_set_rheology: device error");
    if (r->litho_thickness) {
        h->He.swap(He);
        h->D.swap(D);
    }
    if (r->log10_viscosity) {
        h->eta_eff.swap(eta);
        h->R.swap(R);
    }
    return upload_static(h);
}

int fi_set_kernels(fi_handle* h, const double* GE, const double* GN)
{
    if (!h) return FI_E_ARG;
    int rc;
    if (GE) { h->GE.assign(GE, GE + h->n); if ((rc = kernel_spectrum(h, h->GE, 0))) return rc; }
    if (GN) { h->GN.assign(GN, GN + h->n); if ((rc = kernel_spectrum(h, h->GN, 1))) return rc; }
    return FI_OK;
}

int fi_init_ref(fi_handle* h, const double* z_bed, const double* H_ice, double bsl, const double* dz_ss)
{
    // isos_init_ref, src/fastisostasy.f90:550-575
    if (!h || !z_bed || !H_ice) return FI_E_ARG;
    const size_t ni = (size_t)h->nx_ice * h->ny_ice;
    int rc;
    if ((rc = upload(h, h->dH, z_bed, ni * 8))) return rc;
    out2in(h->z_bed_ref, h->dH, h->d, 1e6, 0, h->s);
    CK(cudaStreamSynchronize(h->s));
    if ((rc = upload(h, h->dH, H_ice, ni * 8))) return rc;
    out2in(h->Hice_ref, h->dH, h->d, 0.0, 0, h->s);
    if (dz_ss) { if ((rc = upload(h, h->dz_ss_ref, dz_ss, h->n * 8))) return rc; }
    h->ref_bsl = bsl;
    h->ref_was_set = 1;
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

int fi_init_state(fi_handle* h, const double* z_bed, const double* H_ice, double time, fi_bsl* bsl)
{
    ApiRange nr("fi_init_state");
    // isos_init_state, src/fastisostasy.f90:596-660 (no restart file)
    if (!h || !z_bed || !H_ice || !bsl) return FI_E_ARG;
    const size_t ni = (size_t)h->nx_ice * h->ny_ice;
    const double now_bsl = bsl->bsl_now;
    int rc;
    Dom& d = h->d;
    if ((rc = upload(h, h->dH, z_bed, ni * 8))) return rc;
    out2in(d.z_bed, h->dH, d, 0.0, 1, h->s);
    CK(cudaStreamSynchronize(h->s));
    if ((rc = upload(h, h->dH, H_ice, ni * 8))) return rc;
    out2in(d.Hice, h->dH, d, 0.0, 1, h->s);
    CK(cudaStreamSynchronize(h->s));
    if (!h->ref_was_set) {
        // isos_init_ref(isos, z_bed, H_ice, now%bsl, now%dz_ss)
        if ((rc = fi_init_ref(h, z_bed, H_ice, now_bsl, nullptr))) return rc;
        CK(cudaMemcpyAsync(h->dz_ss_ref, d.dz_ss, h->n * 8, cudaMemcpyDeviceToDevice, h->s));
    }
    // ref%z_ss = ref%bsl + 0 + ref%dz_ss ; now%z_ss = now%bsl + now%z_ss + now%dz_ss ; Haf ; masks
    CK(cudaMemsetAsync(h->z_ss_ref, 0, h->n * 8, h->s));
    state_diag(h->z_ss_ref, h->z_ss_ref, h->dz_ss_ref, h->ref_bsl, h->z_bed_ref, h->Hice_ref, h->Haf_ref, h->mo_ref,
               h->mg_ref, h->mc_ref, h->n, d.rho_sw_over_ice, h->s);
    state_diag(d.z_ss, d.z_ss, d.dz_ss, now_bsl, d.z_bed, d.Hice, d.Haf, d.m_ocean, d.m_grounded, d.m_cont, h->n,
               d.rho_sw_over_ice, h->s);
    h->time_prog = time;
    h->time_diag = time;
    if (h->wrefhi) split_hilo(h->w_ref, h->wrefhi, h->wreflo, h->n, h->s);
    enqueue_args(h, time, bsl, true);
    if ((rc = upload(h, h->dH, H_ice, ni * 8))) return rc;
    // The nested isos_update runs with the ode clock still zero: for time <= 0
    // its integrator loop does not execute; for time > 0 the reference would
    // step with dt = 0, which is skipped here.
    if ((rc = update_any(h, h->dH, time, false))) return rc;
    // ode%dt = dt_init, ode%t = time, ode%x = now%w
    CK(cudaMemcpyAsync(d.x, d.w, h->n * 8, cudaMemcpyDeviceToDevice, h->s));
    Ctl hc;
    CK(cudaMemcpyAsync(&hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    hc.t = time;
    hc.dt = h->p.dt_init;
    hc.done = 0;
    CK(cudaMemcpyAsync(h->ctl, &hc, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    CK(cudaStreamSynchronize(h->s));
    h->h_t = time;
    h->h_dt = h->p.dt_init;
    bsl->bsl_now = hc.bsl;
    h->state_ready = 1;
    Ctl st;
    return read_status(h, &st);
}

namespace {
UpdateClock::UpdateClock(fi_handle* hh) : h(hh), t0(std::chrono::steady_clock::now()) {}
UpdateClock::~UpdateClock()
{
    h->updates++;
    h->host_update_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
}  // namespace

int fi_update_async(fi_handle* h, const double* d_H_ice, double time, fi_bsl* bsl)
{
    ApiRange nr("fi_update_async");
    if (!h || !bsl) return FI_E_ARG;
    UpdateClock uc(h);
    if (!h->state_ready) return fail(h, FI_E_STATE, "fi_update before fi_init_state");
    enqueue_args(h, time, bsl, bsl->method == 0 || bsl->method == 1);
    if (d_H_ice) {
        CK(cudaMemcpyAsync(h->dH, d_H_ice, (size_t)h->nx_ice * h->ny_ice * 8, cudaMemcpyDeviceToDevice, h->s));
    }
    return update_any(h, h->dH, time, true);
}

int fi_set_max_rejections(fi_handle* h, int64_t max_per_update)
{
    if (!h || max_per_update < 0) return FI_E_ARG;
    const long long v = max_per_update ? (long long)max_per_update : kDefaultMaxReject;
    // in stream order: updates already enqueued keep the limit they saw
    CK(cudaMemcpyAsync((char*)h->ctl + offsetof(Ctl, max_reject), &v, sizeof(v), cudaMemcpyHostToDevice, h->s));
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

int fi_metrics_json(fi_handle* h, char* buf, size_t len)
{
    if (!h || !buf || len == 0) return FI_E_ARG;
    Ctl hc;
    CK(cudaMemcpyAsync(&hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    const fi_params& p = h->p;
    const int n = snprintf(buf, len,
                           "{\"nx\": %d, \"ny\": %d, \"nx_ice\": %d, \"ny_ice\": %d, \"precision\": \"%s\", "
                           "\"method\": %d, \"dt_method\": %d, \"stage_mode\": %d, \"step_engine\": %s, "
                           "\"updates\": %lld, \"t\": %.17g, \"dt\": %.17g, \"n_accept\": %lld, \"n_reject\": %lld, "
                           "\"n_attempt\": %lld, \"kernels_enqueued\": %lld, \"graphs_captured\": %d, "
                           "\"host_update_ms\": %.6f, \"status\": %d}",
                           h->nx, h->ny, h->nx_ice, h->ny_ice, mixed(h) ? "mixed" : "fp64", p.method, p.dt_method,
                           p.stage_mode, h->engine_ok ? "true" : "false", h->updates, hc.t, hc.dt, hc.n_accept,
                           hc.n_reject, hc.n_attempt, h->launches, (int)h->graphs.size(), 1e3 * h->host_update_s,
                           hc.status);
    return (n < 0 || (size_t)n >= len) ? FI_E_SIZE : FI_OK;
}

int fi_synchronize(fi_handle* h)
{
    if (!h) return FI_E_ARG;
    Ctl hc;
    return read_status(h, &hc);
}

int fi_update(fi_handle* h, const double* H_ice, double time, fi_bsl* bsl, fi_out* out)
{
    ApiRange nr("fi_update");
    if (!h || !H_ice || !bsl) return FI_E_ARG;
    UpdateClock uc(h);
    if (!h->state_ready) return fail(h, FI_E_STATE, "fi_update before fi_init_state");
    const size_t ni = (size_t)h->nx_ice * h->ny_ice;
    int rc;
    auto pinned = [&](const void* ptr) {
        if (!ptr) return false;
        for (const auto& e : h->pin_seen)
            if (e.p == ptr) return e.pinned;
        const bool pl = host_pinned(ptr);
        h->pin_seen[h->pin_next] = {ptr, pl};
        h->pin_next = (h->pin_next + 1) % 16;
        return pl;
    };
    if (ni >= (1u << 16) && pinned(H_ice)) {
        CK(cudaMemcpyAsync(h->dH, H_ice, ni * 8, cudaMemcpyHostToDevice, h->s));
    } else {
        if (ni < (1u << 16)) memcpy(h->hpin, H_ice, ni * 8);
        else pool_copy(h->hpin, H_ice, ni * 8, 8);
        CK(cudaMemcpyAsync(h->dH, h->hpin, ni * 8, cudaMemcpyHostToDevice, h->s));
    }
    enqueue_args(h, time, bsl, true);
    if ((rc = update_any(h, h->dH, time, true))) return rc;
    const bool piped = out && ni >= (1u << 16);
    double* dst[8] = {nullptr};
    uint8_t* mdst[3] = {nullptr};
    bool direct[11] = {false};   // piped fields copied straight into a page-locked caller array
    if (out) {
        double* d8[8] = {out->z_bed, out->z_ss, out->dz_ss, out->w, out->we, out->dwdt, out->canom_full, out->Hice};
        uint8_t* m3[3] = {out->maskocean, out->maskgrounded, out->maskcontinent};
        for (int f = 0; f < 8; ++f) dst[f] = d8[f];
        for (int f = 0; f < 3; ++f) mdst[f] = m3[f];
        if (piped) {
            for (int f = 0; f < 8; ++f) direct[f] = pinned(dst[f]);
            for (int f = 0; f < 3; ++f) direct[8 + f] = pinned(mdst[f]);
        }
    }
    if (piped && h->ev_field.empty()) {
        h->ev_field.resize(11, nullptr);
        for (auto& e : h->ev_field) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (piped && !h->hctl) CK(cudaMallocHost(&h->hctl, sizeof(Ctl)));
    // piped: the 8 double fields, then the 3 masks as bytes
    uint8_t* const dmask = (uint8_t*)(h->dpack + (size_t)8 * ni);
    uint8_t* const hmask = (uint8_t*)(h->hpin + (size_t)8 * ni);
    if (out) {
        if (piped) {
            gather_bytes(h->gsrc, h->gmsrc, 8, 3, h->d, h->dpack, dmask, h->s);
            // one copy per field, each followed by its event
            for (int f = 0; f < 11; ++f) {
                if (f < 8) {
                    if (!dst[f]) continue;
                    CK(cudaMemcpyAsync(direct[f] ? dst[f] : h->hpin + (size_t)f * ni, h->dpack + (size_t)f * ni,
                                       ni * 8, cudaMemcpyDeviceToHost, h->s));
                } else {
                    if (!mdst[f - 8]) continue;
                    CK(cudaMemcpyAsync(direct[f] ? mdst[f - 8] : hmask + (size_t)(f - 8) * ni,
                                       dmask + (size_t)(f - 8) * ni, ni, cudaMemcpyDeviceToHost, h->s));
                }
                CK(cudaEventRecord(h->ev_field[f], h->s));
            }
        } else {
            gather(h->gsrc, h->gmsrc, 8, 3, h->d, h->dpack, h->s);
            CK(cudaMemcpyAsync(h->hpin, h->dpack, ni * 11 * 8, cudaMemcpyDeviceToHost, h->s));
        }
    }
    Ctl hc;
    if (piped) {
        // the control block last, into page-locked memory: the call does not
        // wait here, and the unpack below follows the field copies
        CK(cudaMemcpyAsync(h->hctl, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    } else {
        rc = read_status(h, &hc);
        bsl->bsl_now = hc.bsl;
    }
    if (out) {
        // the staged fields into the caller's arrays, each field in kParts
        // slices spread over the host pool (a single core copies a few GB/s;
        // the fields are ~100 B per cell, and 11 whole-field tasks left the
        // pool's threads waiting on the last few)
        constexpr int kParts = 4;
        const size_t chunk = (ni + kParts - 1) / kParts;
        auto copy_part = [&](int t) {
            const int f = t / kParts;
            const size_t a = (size_t)(t % kParts) * chunk, b = std::min(ni, a + chunk);
            if (a >= b || direct[f]) return;
            if (f < 8 ? !dst[f] : !mdst[f - 8]) return;
            if (piped) cudaEventSynchronize(h->ev_field[f]);
            if (f < 8) {
                if (dst[f]) memcpy(dst[f] + a, h->hpin + (size_t)f * ni + a, (b - a) * 8);
            } else if (mdst[f - 8]) {
                if (piped) {
                    memcpy(mdst[f - 8] + a, hmask + (size_t)(f - 8) * ni + a, b - a);
                } else {
                    const double* src = h->hpin + (size_t)f * ni;
                    uint8_t* m = mdst[f - 8];
                    for (size_t e = a; e < b; ++e) m[e] = src[e] != 0.0;
                }
            }
        };
        if (ni < (1u << 16)) {
            for (int t = 0; t < 11 * kParts; ++t) copy_part(t);
        } else {
            HostPool::get().run(11 * kParts, copy_part);
        }
    }
    if (piped) {
        CK(cudaStreamSynchronize(h->s));
        hc = *h->hctl;
        rc = decode_status(h, &hc);
        bsl->bsl_now = hc.bsl;
    }
    return rc;
}

int fi_bsl_update(fi_bsl* b, double year_bp)
{
    // bsl_update, src/barysealevel.f90:195-252 (series from caller tables)
    if (!b) return FI_E_ARG;
    auto interp = [](const double* x, const double* y, int n, double xo) {
        if (xo < x[0]) return y[0];
        if (xo > x[n - 1]) return y[n - 1];
        int j = 0;
        while (j < n && !(x[j] >= xo)) ++j;
        if (j == 0) return y[0];
        if (j == n) return y[n - 1];
        const double a = (xo - x[j - 1]) / (x[j] - x[j - 1]);
        return y[j - 1] + a * (y[j] - y[j - 1]);
    };
    b->time = year_bp;
    switch (b->method) {
    case 0: b->bsl_now = b->bsl_init; break;
    case 1:
        if (b->n_series < 1) return FI_E_ARG;
        b->bsl_now = interp(b->series_t, b->series_v, b->n_series, year_bp);
        break;
    case 3:
        if (b->n_series < 1) return FI_E_ARG;
        b->bsl_now = interp(b->series_t, b->series_v, b->n_series, year_bp);
        /* fall through */
    case 2:
        if (b->constant_ocean_surface || b->n_aocean <= 0) b->A_ocean_now = b->A_ocean_pd;
        else b->A_ocean_now = interp(b->bsl_vec, b->aocean_vec, b->n_aocean, b->bsl_now);
        break;
    default: return FI_E_ARG;
    }
    return FI_OK;
}

int fi_get_field(fi_handle* h, int which, double* out)
{
    if (!h || !out) return FI_E_ARG;
    const size_t n = h->n;
    const Dom& d = h->d;
    const double* src = nullptr;
    const uint8_t* msk = nullptr;
    const std::vector<double>* hv = nullptr;
    switch (which) {
    case FI_FIELD_Z_BED: src = d.z_bed; break;
    case FI_FIELD_DWDT: src = d.dwdt; break;
    case FI_FIELD_W: src = d.w; break;
    case FI_FIELD_WE: src = d.we; break;
    case FI_FIELD_HAF: src = d.Haf; break;
    case FI_FIELD_HICE: src = d.Hice; break;
    case FI_FIELD_Z_SS: src = d.z_ss; break;
    case FI_FIELD_DZ_SS: src = d.dz_ss; break;
    case FI_FIELD_CANOM_LOAD: src = d.c_load; break;
    case FI_FIELD_CANOM_FULL: src = d.c_full; break;
    case FI_FIELD_MASS_ANOM: src = d.mass; break;
    case FI_FIELD_MASKOCEAN: msk = d.m_ocean; break;
    case FI_FIELD_MASKGROUNDED: msk = d.m_grounded; break;
    case FI_FIELD_MASKCONTINENT: msk = d.m_cont; break;
    case FI_FIELD_CANOM_MANTLE: src = d.c_mantle; break;
    case FI_FIELD_CANOM_LITHO: src = d.c_litho; break;
    case FI_FIELD_CANOM_SEAWATER: src = d.c_sw; break;
    case FI_FIELD_CANOM_ICE: src = d.c_ice; break;
    case FI_FIELD_X: src = d.x; break;
    case FI_FIELD_KAPPA: hv = &h->kappa; break;
    case FI_FIELD_D_LITH: hv = &h->D; break;
    case FI_FIELD_ETA_EFF: hv = &h->eta_eff; break;
    case FI_FIELD_R: hv = &h->R; break;
    case FI_FIELD_MASKACTIVE: msk = d.mactive; break;
    case FI_FIELD_GE: hv = &h->GE; break;
    case FI_FIELD_GN: hv = &h->GN; break;
    default: return fail(h, FI_E_ARG, "unknown field %d", which);
    }
    if (hv) { memcpy(out, hv->data(), n * 8); return FI_OK; }
    if (src) {
        CK(cudaMemcpyAsync(out, src, n * 8, cudaMemcpyDeviceToHost, h->s));
        CK(cudaStreamSynchronize(h->s));
        return FI_OK;
    }
    std::vector<uint8_t> m(n);
    CK(cudaMemcpyAsync(m.data(), msk, n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    for (size_t e = 0; e < n; ++e) out[e] = m[e];
    return FI_OK;
}

int fi_get_scalars(fi_handle* h, double* o)
{
    if (!h || !o) return FI_E_ARG;
    Ctl hc;
    CK(cudaMemcpyAsync(&hc, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    o[0] = hc.t; o[1] = hc.dt; o[2] = h->time_diag; o[3] = hc.bsl; o[4] = hc.V_af; o[5] = hc.V_den;
    o[6] = hc.deltaV; o[7] = hc.dbsl_total; o[8] = 0.0; o[9] = (double)hc.n_accept; o[10] = (double)hc.n_reject;
    o[11] = h->spy; o[12] = h->cc; o[13] = h->Vden; o[14] = (double)h->Px; o[15] = h->ref_bsl;
    return FI_OK;
}

int fi_lvelva(fi_handle* h, const double* w, const double* canom_full, double* dwdt)
{
    if (!h || !w || !canom_full || !dwdt) return FI_E_ARG;
    const size_t n = h->n;
    int rc;
    double* tmp;
    if ((rc = dalloc(h, &tmp, n * 8))) return rc;
    if ((rc = upload(h, h->y, w, n * 8)) || (rc = upload(h, tmp, canom_full, n * 8))) return rc;
    if (mixed(h)) {
        q0_from_cf<float>((float*)h->q0, tmp, h->d.mactive, h->p.g, n, h->s);
        if (h->p.method == 3 && h->fc.dxm == nullptr) {
            // uniform spacing: w as a float pair through the column-strip
            // stencil, as the mixed reference-compatible Tsit5 evaluates it
            float* pair;
            if ((rc = dalloc(h, &pair, 2 * n * sizeof(float)))) return rc;
            split_hilo(h->y, pair, pair + n, n, h->s);
            rhs<float>(h, h->y, nullptr, (float*)h->raw[0], nullptr, pair, pair + n);
        } else {
            rhs<float>(h, h->y, nullptr, (float*)h->raw[0]);
        }
        rhs_finish<float>(tmp, (const float*)h->raw[0], h->nx, h->ny, h->spy, h->s);
    } else {
        q0_from_cf<double>((double*)h->q0, tmp, h->d.mactive, h->p.g, n, h->s);
        rhs<double>(h, h->y, nullptr, (double*)h->raw[0]);
        rhs_finish<double>(tmp, (const double*)h->raw[0], h->nx, h->ny, h->spy, h->s);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dwdt, tmp, n * 8, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    // release the temporaries (tmp, and the float pair when one was made)
    while (!h->allocs.empty() && h->allocs.back() != (void*)tmp) {
        cudaFree(h->allocs.back());
        h->allocs.pop_back();
    }
    h->allocs.pop_back();
    cudaFree(tmp);
    return FI_OK;
}

int fi_convolve(fi_handle* h, int kernel, const double* in, double* out)
{
    if (!h || !in || !out || kernel < 0 || kernel > 1) return FI_E_ARG;
    const size_t n = h->n;
    int rc;
    if ((rc = upload(h, h->we_raw, in, n * 8))) return rc;
    if (mixed(h)) {
        cast_from_double<float>((float*)h->conv_in, h->we_raw, n, h->s);
        conv<float>(h, kernel, h->dz_raw, h->corners);
    } else {
        cast_from_double<double>((double*)h->conv_in, h->we_raw, n, h->s);
        conv<double>(h, kernel, h->dz_raw, h->corners);
    }
    sub_corner(h->we_raw, h->dz_raw, h->corners, n, h->s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, h->we_raw, n * 8, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

// ---- restart: device state <-> flat double buffer ---------------------------
namespace {
struct StateView {
    std::vector<double*> f;
    std::vector<uint8_t*> m;
};
StateView state_view(fi_handle* h)
{
    Dom& d = h->d;
    StateView v;
    v.f = {d.z_bed, d.w, d.we, d.Haf, d.Hice, d.z_ss, d.dz_ss, d.dwdt, d.x, d.c_ice, d.c_sw, d.c_litho,
           d.c_mantle, d.c_load, d.c_full, d.mass, h->z_bed_ref, h->Hice_ref, h->Haf_ref, h->z_ss_ref, h->we_ref,
           h->w_ref, h->dz_ss_ref};
    v.m = {d.m_ocean, d.m_grounded, d.m_cont};
    return v;
}
const size_t kScalarSlots = 8 + sizeof(Ctl) / sizeof(double) + 1;
}  // namespace

size_t fi_state_size(const fi_handle* h)
{
    if (!h) return 0;
    return (23 + 3) * h->n + kScalarSlots;
}

int fi_state_export(fi_handle* h, double* buf)
{
    if (!h || !buf) return FI_E_ARG;
    StateView v = state_view(h);
    const size_t n = h->n;
    size_t off = 0;
    for (double* p : v.f) { CK(cudaMemcpyAsync(buf + off, p, n * 8, cudaMemcpyDeviceToHost, h->s)); off += n; }
    std::vector<uint8_t> m(n);
    for (uint8_t* p : v.m) {
        CK(cudaMemcpyAsync(m.data(), p, n, cudaMemcpyDeviceToHost, h->s));
        CK(cudaStreamSynchronize(h->s));
        for (size_t e = 0; e < n; ++e) buf[off + e] = m[e];
        off += n;
    }
    double* s = buf + off;
    s[0] = h->time_diag; s[1] = h->time_prog; s[2] = h->h_t; s[3] = h->h_dt; s[4] = h->ref_bsl;
    s[5] = h->ref_was_set; s[6] = h->state_ready; s[7] = 0.0;
    CK(cudaMemcpyAsync(s + 8, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

int fi_state_import(fi_handle* h, const double* buf)
{
    if (!h || !buf) return FI_E_ARG;
    StateView v = state_view(h);
    const size_t n = h->n;
    size_t off = 0;
    for (double* p : v.f) { CK(cudaMemcpyAsync(p, buf + off, n * 8, cudaMemcpyHostToDevice, h->s)); off += n; }
    CK(cudaStreamSynchronize(h->s));
    std::vector<uint8_t> m(n);
    for (uint8_t* p : v.m) {
        for (size_t e = 0; e < n; ++e) m[e] = buf[off + e] != 0.0;
        CK(cudaMemcpyAsync(p, m.data(), n, cudaMemcpyHostToDevice, h->s));
        CK(cudaStreamSynchronize(h->s));
        off += n;
    }
    const double* s = buf + off;
    h->time_diag = s[0]; h->time_prog = s[1]; h->h_t = s[2]; h->h_dt = s[3]; h->ref_bsl = s[4];
    h->ref_was_set = (int)s[5]; h->state_ready = (int)s[6];
    if (h->wrefhi) split_hilo(h->w_ref, h->wrefhi, h->wreflo, h->n, h->s);
    CK(cudaMemcpyAsync(h->ctl, s + 8, sizeof(Ctl), cudaMemcpyHostToDevice, h->s));
    CK(cudaStreamSynchronize(h->s));
    return FI_OK;
}

}  // extern "C"

// ---- batched ensembles ------------------------------------------------------
// One update of every member as a single CUDA graph: the per-member update
// head (sea level, masks, loads, convolutions) as parallel branches, then
// one WHILE loop of batched Tsit5 attempts over all members (one launch per
// pass for the whole ensemble), then the per-member update tails.
struct fi_batch {
    std::vector<fi_handle*> hs;
    bool mixed = false;
    int nm = 0;
    cudaStream_t s = nullptr, s_body = nullptr;
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev;
    BMember* dM = nullptr;
    int* doff = nullptr;                 // 4 x (nm + 1): flexure, rows, columns, reductions
    int* dcl = nullptr;                  // compacted lists of the current attempt (blist_ints(nm))
    int nblk[4] = {0, 0, 0, 0};          // virtual blocks per phase (all members)
    int grid[4] = {0, 0, 0, 0};          // resident grid per phase
    int rows_threads = 32, cols_threads = 32;
    size_t rows_smem = 0, cols_smem = 0;
    static constexpr int kRing = 4;
    BArgs* hargs[kRing] = {nullptr, nullptr, nullptr, nullptr};   // pinned
    BArgs* dargs[kRing] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t args_ev[kRing] = {nullptr, nullptr, nullptr, nullptr};
    int ring = 0;
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    int seen[2] = {0, 0};
    long long launches = 0;
    int* dmore = nullptr;                // loop condition of the eager path
    bool eager = false;
    bool true_stages = false;            // members run Tsit5 with true stages (stage_mode 1)
    std::vector<BMember> hM;             // host copy of the member descriptors
    std::vector<int> hoff;               // host copy of the virtual-block offsets (4 x (nm + 1))
    int shape[4] = {0, 0, 16, 8};        // rows / columns per transform block (0: single-domain shape), strip rows, waves
};

// Per-member transform and stencil shapes, the virtual-block offsets and
// the resident grids of the batched launches; uploads the descriptors.
// RB / CB <= 0: the single-domain shapes.
int batch_shape(fi_batch* b, int RB, int CB, int fseg, int waves)
{
    const int n = b->nm;
    std::vector<int> off(4 * (n + 1), 0);
    const size_t c2 = b->mixed ? sizeof(float2) : sizeof(double2);
    b->rows_threads = b->cols_threads = 0;
    b->rows_smem = b->cols_smem = 0;
    for (int i = 0; i < n; ++i) {
        BMember& m = b->hM[i];
        m.RB = RB > 0 ? RB : rhs_rows_per_block(m.p.h);
        m.CB = CB > 0 ? CB : (b->mixed ? rhs_cols_per_block<float>(m.p.ny) : rhs_cols_per_block<double>(m.p.ny));
        m.fseg = fseg;
        const int fblk = (b->mixed && (!b->true_stages || m.yhi)) ? batch_flexure_blocks(m.p.nx, m.p.ny, m.fseg)
                                                                  : m.fgx * ((m.p.ny + 7) / 8);
        const int rblk = (m.p.ny + m.RB - 1) / m.RB;
        const int cblk = (m.p.h + 1 + m.CB - 1) / m.CB;
        off[i + 1] = off[i] + fblk;
        off[(n + 1) + i + 1] = off[(n + 1) + i] + rblk;
        off[2 * (n + 1) + i + 1] = off[2 * (n + 1) + i] + cblk;
        off[3 * (n + 1) + i + 1] = off[3 * (n + 1) + i] + m.red_nblk;
        const int rt = rhs_threads_for(m.RB * m.p.h / 4), ct = rhs_threads_for(m.CB * m.p.ny / 4);
        if (rt > b->rows_threads) b->rows_threads = rt;
        if (ct > b->cols_threads) b->cols_threads = ct;
        const size_t rs = 2 * (size_t)m.RB * m.p.h * c2, cs = 2 * (size_t)m.CB * (m.p.ny + 1) * c2;   // padded columns
        if (rs > b->rows_smem) b->rows_smem = rs;
        if (cs > b->cols_smem) b->cols_smem = cs;
    }
    if (b->rows_smem > 200 * 1024 || b->cols_smem > 200 * 1024) return 2;   // shape does not fit
    for (int k = 0; k < 4; ++k) b->nblk[k] = off[k * (n + 1) + n];
    b->hoff = off;
    // on the batch stream that reads them (a plain cudaMemcpy from pageable
    // memory is not ordered before work on a non-blocking stream)
    if (cudaMemcpyAsync(b->dM, b->hM.data(), n * sizeof(BMember), cudaMemcpyHostToDevice, b->s) != cudaSuccess ||
        cudaMemcpyAsync(b->doff, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, b->s) != cudaSuccess ||
        cudaStreamSynchronize(b->s) != cudaSuccess)
        return 1;
    int res[4];
    if (b->mixed) {
        batch_prepare<float>(b->rows_smem, b->cols_smem);
        batch_grids<float>(b->rows_smem, b->cols_smem, b->rows_threads, b->cols_threads, &res[0], &res[1], &res[2],
                           &res[3]);
    } else {
        batch_prepare<double>(b->rows_smem, b->cols_smem);
        batch_grids<double>(b->rows_smem, b->cols_smem, b->rows_threads, b->cols_threads, &res[0], &res[1], &res[2],
                            &res[3]);
    }
    // resident grid times `waves`, at most one block per virtual block
    for (int k = 0; k < 4; ++k) {
        const long long g = waves > 0 ? (long long)res[k] * waves : (long long)b->nblk[k];
        b->grid[k] = (int)(g < b->nblk[k] ? g : b->nblk[k]);
        if (b->grid[k] < 1) b->grid[k] = 1;
    }
    b->shape[0] = RB;
    b->shape[1] = CB;
    b->shape[2] = fseg;
    b->shape[3] = waves;
    return 0;
}

namespace {

// One Tsit5 attempt of every member that still has one, as batched launches.
template <typename T> void batch_attempt(fi_batch* b, cudaStream_t s, cudaGraphConditionalHandle loop, int* more_out)
{
    const int nm = b->nm;
    const int* off = b->doff;
    batch_attempt_begin(b->dM, nm, kMaxAttempts, off, b->dcl, s);
    const BList LF = blist(b->dcl, nm, 0), LR = blist(b->dcl, nm, 1), LC = blist(b->dcl, nm, 2),
                LT = blist(b->dcl, nm, 3);
    if (b->true_stages) {
        // Dormand-Prince 5(4) with FSAL (tsit_true_attempt per member): k_0
        // where no accepted attempt left it cached, then stages 1-6 for every
        // member with an attempt, the embedded error, decision, commit, FSAL
        const BList LF6 = blist(b->dcl, nm, 4), LR6 = blist(b->dcl, nm, 5), LC6 = blist(b->dcl, nm, 6);
        batch_flexure_y<T>(b->dM, LF, b->grid[0], 0, s);
        batch_rows_fwd<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, s);
        batch_cols_hartley<T>(b->dM, LC, b->grid[2], b->cols_threads, b->cols_smem, s);
        batch_rows_inv<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, s, 0);
        for (int i = 1; i <= 6; ++i) {
            batch_dp_stage<T>(b->dM, LT, b->grid[3], i, s);
            batch_flexure_y<T>(b->dM, LF6, b->grid[0], i, s);
            batch_rows_fwd<T>(b->dM, LR6, b->grid[1], b->rows_threads, b->rows_smem, s);
            batch_cols_hartley<T>(b->dM, LC6, b->grid[2], b->cols_threads, b->cols_smem, s);
            batch_rows_inv<T>(b->dM, LR6, b->grid[1], b->rows_threads, b->rows_smem, s, i);
        }
        batch_dp_err<T>(b->dM, LT, b->grid[3], s);
        batch_ts_err<T>(b->dM, LT, b->grid[3], s);
        batch_ts_commit<T>(b->dM, LT, b->grid[3], s);
        batch_fsal<T>(b->dM, LT, b->grid[3], s);
        batch_attempt_end(b->dM, nm, loop, s, more_out, 1);
        b->launches += 40;
        return;
    }
    batch_flexure<T>(b->dM, LF, b->grid[0], s);
    batch_rows_fwd<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, s);
    batch_cols_hartley<T>(b->dM, LC, b->grid[2], b->cols_threads, b->cols_smem, s);
    batch_rows_inv<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, s);
    if (sizeof(T) == 4) {
        // mixed members always carry now%w's float pair
        batch_ts_fused(b->dM, LT, b->grid[3], s);
        batch_ts_commit_pair(b->dM, LT, b->grid[3], s);
        b->launches += 9;
    } else {
        batch_ts_max<T>(b->dM, LT, b->grid[3], s);
        batch_ts_err<T>(b->dM, LT, b->grid[3], s);
        batch_ts_commit<T>(b->dM, LT, b->grid[3], s);
        b->launches += 10;
    }
    batch_attempt_end(b->dM, nm, loop, s, more_out);
}

// The same update without a graph: the host reads the loop condition after
// every attempt (profiling; FI_BATCH_EAGER=1).
template <typename T> int batch_eager(fi_batch* b, bool diag)
{
    auto fork_join = [&](auto&& body) -> int {
        if (cudaEventRecord(b->ev_fork, b->s) != cudaSuccess) return FI_E_CUDA;
        for (int i = 0; i < b->nm; ++i) {
            fi_handle* h = b->hs[i];
            if (cudaStreamWaitEvent(h->s, b->ev_fork, 0) != cudaSuccess) return FI_E_CUDA;
            body(h);
            if (cudaEventRecord(b->ev[i], h->s) != cudaSuccess) return FI_E_CUDA;
            if (cudaStreamWaitEvent(b->s, b->ev[i], 0) != cudaSuccess) return FI_E_CUDA;
        }
        return FI_OK;
    };
    int rc = fork_join([&](fi_handle* h) {
        enqueue_pre<T>(h, h->dH, diag, true);
        if (h->d.whi) split_hilo(h->d.w, h->d.whi, h->d.wlo, h->n, h->s);
        if (h->yhi) split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, h->s);
    });
    if (rc) return rc;
    batch_loop_begin(b->dM, b->nm, b->s);
    for (long long it = 0;; ++it) {
        batch_attempt<T>(b, b->s, 0, b->dmore);
        int more = 0;
        if (cudaMemcpyAsync(&more, b->dmore, sizeof(int), cudaMemcpyDeviceToHost, b->s) != cudaSuccess ||
            cudaStreamSynchronize(b->s) != cudaSuccess)
            return FI_E_CUDA;
        if (!more) break;
        if (it > kMaxAttempts) return FI_E_STEP;
    }
    return fork_join([&](fi_handle* h) { enqueue_post<T>(h, (T*)h->raw[0], -1); });
}

template <typename T> int batch_capture(fi_batch* b, bool diag, cudaGraph_t* out)
{
    fi_handle* h0 = b->hs[0];
    const fi_params& p0 = h0->p;
    auto ck = [&](cudaError_t e) { return e == cudaSuccess ? FI_OK : FI_E_CUDA; };
    int rc;
    if ((rc = ck(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal)))) return rc;
    auto join_members = [&](auto&& body) -> int {
        if (cudaEventRecord(b->ev_fork, b->s) != cudaSuccess) return FI_E_CUDA;
        for (int i = 0; i < b->nm; ++i) {
            fi_handle* h = b->hs[i];
            if (cudaStreamWaitEvent(h->s, b->ev_fork, 0) != cudaSuccess) return FI_E_CUDA;
            body(h);
            if (cudaEventRecord(b->ev[i], h->s) != cudaSuccess) return FI_E_CUDA;
            if (cudaStreamWaitEvent(b->s, b->ev[i], 0) != cudaSuccess) return FI_E_CUDA;
        }
        return FI_OK;
    };
    rc = join_members([&](fi_handle* h) {
        enqueue_pre<T>(h, h->dH, diag, true);
        if (h->d.whi) split_hilo(h->d.w, h->d.whi, h->d.wlo, h->n, h->s);
        if (h->yhi) split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, h->s);
    });
    if (!rc) {
        batch_loop_begin(b->dM, b->nm, b->s);
        cudaStreamCaptureStatus st;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaGraphConditionalHandle loop;
        cudaGraphNode_t node;
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        if (cudaStreamGetCaptureInfo(b->s, &st, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
            cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
            rc = FI_E_CUDA;
        } else {
            cp.conditional.handle = loop;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp) != cudaSuccess ||
                cudaStreamUpdateCaptureDependencies(b->s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) !=
                    cudaSuccess ||
                cudaStreamBeginCaptureToGraph(b->s_body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                rc = FI_E_CUDA;
            } else {
                batch_attempt<T>(b, b->s_body, loop, nullptr);
                cudaGraph_t body_out = nullptr;
                if (cudaStreamEndCapture(b->s_body, &body_out) != cudaSuccess) rc = FI_E_CUDA;
            }
        }
    }
    if (!rc) rc = join_members([&](fi_handle* h) { enqueue_post<T>(h, (T*)h->raw[0], -1); });
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->s, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc ? rc : FI_E_CUDA;
    }
    (void)p0;
    *out = graph;
    return FI_OK;
}

void batch_free(fi_batch* b)
{
    for (auto& g : b->g)
        if (g) cudaGraphExecDestroy(g);
    if (b->s) cudaStreamSynchronize(b->s);
    cudaFree(b->dM);
    cudaFree(b->doff);
    cudaFree(b->dcl);
    cudaFree(b->dmore);
    for (int i = 0; i < fi_batch::kRing; ++i) {
        if (b->hargs[i]) cudaFreeHost(b->hargs[i]);
        cudaFree(b->dargs[i]);
        if (b->args_ev[i]) cudaEventDestroy(b->args_ev[i]);
    }
    for (auto e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->s) cudaStreamDestroy(b->s);
    if (b->s_body) cudaStreamDestroy(b->s_body);
    delete b;
}

}  // namespace

int fi_batch_create(fi_handle* const* hs, int n, fi_batch** out)
{
    if (!hs || n < 1 || n > 2048 || !out) return FI_E_ARG;   // the attempt-begin kernel keeps 5 ints per member in shared memory
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        fi_handle* h = hs[i];
        if (!h) return FI_E_ARG;
        if (!h->state_ready) return fail(h, FI_E_STATE, "fi_batch_create before fi_init_state");
        const fi_handle* h0 = hs[0];
        if (h->p.method != 3 || h->p.dt_method != 2 || h->p.stage_mode != h0->p.stage_mode || mixed(h) != mixed(h0) ||
            (mixed(h) && h->p.stage_mode == 0 && !h->d.whi) || (mixed(h) && h->fc.dxm != nullptr) ||
            h->p.dt_diagnostics != h0->p.dt_diagnostics || h->time_diag != h0->time_diag || !h->tsit_graph_ok)
            return fail(h, FI_E_CONFIG,
                        "batched members must run tsit54 with the same stage mode and precision, in lockstep "
                        "(mixed members with uniform spacing)");
    }
    fi_batch* b = new fi_batch();
    b->hs.assign(hs, hs + n);
    b->nm = n;
    b->mixed = mixed(hs[0]);
    b->true_stages = hs[0]->p.stage_mode == 1;
    std::vector<BMember> M(n);
    for (int i = 0; i < n; ++i) {
        fi_handle* h = hs[i];
        BMember& m = M[i];
        memset(&m, 0, sizeof(m));
        m.p = h->prhs;
        m.fc = h->fc;
        m.fcf = flex_coef_f32(h->fc);
        m.norm_scale = 1.0 / (double)(float)((long long)h->prhs.nx * h->prhs.ny);   // nx*ny*1. (default real)
        m.norm_scale_f = (float)m.norm_scale;
        m.y = h->d.w;
        m.q0 = h->q0;
        m.mask = h->d.mactive;
        m.D = h->Dt;
        m.inv2eta = h->inv2eta;
        m.f = h->f;
        m.S = h->S;
        m.mA = h->mA;
        m.mB = h->mB;
        m.raw = h->raw[0];
        for (int q = 0; q < 7; ++q) m.raw7[q] = h->raw[q];
        m.yst = h->y;
        m.wref = h->w_ref;
        if (h->yhi) {
            m.xhi = h->xhi; m.xlo = h->xlo; m.xdw = h->dxw;
            m.yhi = h->yhi; m.ylo = h->ylo; m.ydw = h->ydw;
            m.wrhi = h->wrefhi; m.wrlo = h->wreflo;
        }
        m.even = h->even;
        m.fgx = (m.p.nx + 31) / 32;
        m.red_nblk = ts_grid(h->n);
        m.d = h->d;
        m.atol = h->p.atol;
        m.rtol = h->p.rtol;
        m.q = h->p.q;
        m.dt_max = h->p.dt_max;
    }
    bool ok = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&b->s_body, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&b->dM, n * sizeof(BMember)) == cudaSuccess &&
              cudaMalloc(&b->doff, 4 * (size_t)(n + 1) * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&b->dcl, blist_ints(n) * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&b->dmore, sizeof(int)) == cudaSuccess;
    if (const char* e = getenv("FI_BATCH_EAGER")) b->eager = (e[0] == '1');
    b->ev.assign(n, nullptr);
    for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&b->ev[i], cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; ok && i < fi_batch::kRing; ++i)
        ok = cudaMallocHost(&b->hargs[i], n * sizeof(BArgs)) == cudaSuccess &&
             cudaMalloc(&b->dargs[i], n * sizeof(BArgs)) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->args_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        batch_free(b);
        return FI_E_OOM;
    }
    b->hM.swap(M);
    // default shapes: 8 rows / 8 spectrum columns per transform block for
    // mixed batches (64-byte column segments), 16-row strip tasks, 8 waves;
    // FI_BATCH_RB / FI_BATCH_CB / FI_BATCH_WAVES override (tuning)
    int RB = b->mixed ? 8 : 0, CB = b->mixed ? 8 : 0, waves = 8;
    if (const char* e = getenv("FI_BATCH_RB")) { const int v = atoi(e); if (v >= 1 && v <= 16) RB = v; }
    if (const char* e = getenv("FI_BATCH_CB")) { const int v = atoi(e); if (v >= 1 && v <= 16) CB = v; }
    if (const char* e = getenv("FI_BATCH_WAVES")) waves = atoi(e);
    if (batch_shape(b, RB, CB, 16, waves)) {
        batch_free(b);
        return FI_E_CUDA;
    }
    *out = b;
    return FI_OK;
}

namespace {

// Lists of all members (every list kind) for timing the batched passes.
int batch_all_lists(fi_batch* b)
{
    const int n = b->nm;
    std::vector<int> cl(blist_ints(n), 0);
    cl[0] = cl[1] = n;
    for (int i = 0; i < n; ++i) cl[2 + i] = cl[2 + n + i] = i;
    for (int k = 0; k < 7; ++k) {
        const int src = k < 3 ? k : (k == 3 ? 3 : k - 4);
        for (int i = 0; i <= n; ++i) cl[2 + 2 * n + k * (n + 1) + i] = b->hoff[src * (n + 1) + i];
    }
    return (cudaMemcpyAsync(b->dcl, cl.data(), cl.size() * sizeof(int), cudaMemcpyHostToDevice, b->s) == cudaSuccess &&
            cudaStreamSynchronize(b->s) == cudaSuccess)
               ? 0
               : 1;
}

// Device time [ms] of the first RHS of an attempt over all members: part 1
// the stencil, 2 the row transforms, 3 the column transform, 0 all; best of
// `reps` after one warm-up.
template <typename T> float batch_time_rhs(fi_batch* b, int part, int reps)
{
    const int nm = b->nm;
    const BList LF = blist(b->dcl, nm, 0), LR = blist(b->dcl, nm, 1), LC = blist(b->dcl, nm, 2);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r <= reps; ++r) {
        cudaEventRecord(e0, b->s);
        if (part == 0 || part == 1) {
            if (b->true_stages) batch_flexure_y<T>(b->dM, LF, b->grid[0], 0, b->s);
            else batch_flexure<T>(b->dM, LF, b->grid[0], b->s);
        }
        if (part == 0 || part == 2) batch_rows_fwd<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, b->s);
        if (part == 0 || part == 3) batch_cols_hartley<T>(b->dM, LC, b->grid[2], b->cols_threads, b->cols_smem, b->s);
        if (part == 0 || part == 2) batch_rows_inv<T>(b->dM, LR, b->grid[1], b->rows_threads, b->rows_smem, b->s, 0);
        cudaEventRecord(e1, b->s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cudaGetLastError() == cudaSuccess ? best : -1.f;
}

}  // namespace

int fi_batch_autotune(fi_batch* b, int32_t* chosen4)
{
    if (!b) return FI_E_ARG;
    if (b->seen[0] || b->seen[1]) return FI_E_STATE;
    for (fi_handle* h : b->hs)
        if (cudaStreamSynchronize(h->s) != cudaSuccess) return FI_E_CUDA;
    // the stencil of the reference stages reads now%w's float pair
    for (fi_handle* h : b->hs) {
        if (h->d.whi) split_hilo(h->d.w, h->d.whi, h->d.wlo, h->n, b->s);
        if (h->yhi) split_hilo_dxw(h->d.x, h->xhi, h->xlo, h->wrefhi, h->wreflo, h->dxw, h->n, b->s);
    }
    auto time_of = [&](int part) { return b->mixed ? batch_time_rhs<float>(b, part, 3) : batch_time_rhs<double>(b, part, 3); };
    int sh[4] = {b->shape[0], b->shape[1], b->shape[2], b->shape[3]};
    auto try_shape = [&](const int* c, int part, float* t) -> int {
        const int rc = batch_shape(b, c[0], c[1], c[2], c[3]);
        if (rc == 2) { *t = 1e30f; return 0; }   // does not fit
        if (rc || batch_all_lists(b)) return 1;
        *t = time_of(part);
        return *t < 0 ? 1 : 0;
    };
    // coordinate descent: stencil rows per task, transform rows, transform
    // columns, then waves over the whole RHS
    const int seg_c[3] = {8, 16, 32}, rb_c[4] = {2, 4, 8, 16}, cb_c[5] = {1, 2, 4, 8, 16}, wv_c[4] = {2, 4, 8, 16};
    struct Axis { int idx, part, nc; const int* c; };
    const Axis axes[4] = {{2, 1, 3, seg_c}, {0, 2, 4, rb_c}, {1, 3, 5, cb_c}, {3, 0, 4, wv_c}};
    for (const Axis& ax : axes) {
        if (ax.idx == 2 && (!b->mixed || b->true_stages)) continue;   // column strips: mixed reference stages only
        int best_v = sh[ax.idx];
        float best_t = 1e30f;
        for (int k = 0; k < ax.nc; ++k) {
            int c[4] = {sh[0], sh[1], sh[2], sh[3]};
            c[ax.idx] = ax.c[k];
            float t;
            if (try_shape(c, ax.part, &t)) return FI_E_CUDA;
            if (t < best_t) { best_t = t; best_v = ax.c[k]; }
        }
        sh[ax.idx] = best_v;
    }
    if (batch_shape(b, sh[0], sh[1], sh[2], sh[3])) return FI_E_CUDA;
    if (cudaStreamSynchronize(b->s) != cudaSuccess) return FI_E_CUDA;
    if (chosen4)
        for (int k = 0; k < 4; ++k) chosen4[k] = sh[k];
    return FI_OK;
}

int fi_batch_set_priority(fi_batch* b, int level)
{
    if (!b || level < 0 || level > 1) return FI_E_ARG;
    if (b->seen[0] || b->seen[1]) return FI_E_STATE;
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return FI_E_CUDA;
    cudaStream_t ns = nullptr;
    if (cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, level ? greatest : least) != cudaSuccess)
        return FI_E_CUDA;
    if (cudaStreamSynchronize(b->s) != cudaSuccess) {
        cudaStreamDestroy(ns);
        return FI_E_CUDA;
    }
    cudaStreamDestroy(b->s);
    b->s = ns;
    return FI_OK;
}

int fi_batch_step(fi_batch* b, double time, fi_bsl* bsl)
{
    ApiRange nr("fi_batch_step");
    if (!b || !bsl) return FI_E_ARG;
    fi_handle* h0 = b->hs[0];
    const bool diag = time - h0->time_diag >= sp(1e-3);   // the same for every member (lockstep)
    const int key = diag ? 1 : 0;
    if (!b->seen[key]) {
        // first update of this kind: each member on its own path (sets kernel
        // attributes and per-handle graphs), then the batch stream joins
        b->seen[key] = 1;
        for (int i = 0; i < b->nm; ++i) {
            if (int rc = fi_update_async(b->hs[i], nullptr, time, &bsl[i])) return rc;
            if (cudaEventRecord(b->ev[i], b->hs[i]->s) != cudaSuccess ||
                cudaStreamWaitEvent(b->s, b->ev[i], 0) != cudaSuccess)
                return FI_E_CUDA;
        }
        return FI_OK;
    }
    // host side of isos_update for every member (src/fastisostasy.f90:782-787)
    BArgs* ha = b->hargs[b->ring];
    if (cudaEventSynchronize(b->args_ev[b->ring]) != cudaSuccess) return FI_E_CUDA;   // ring slot free
    for (int i = 0; i < b->nm; ++i) {
        fi_handle* h = b->hs[i];
        if (diag) h->time_diag = h->time_diag + h->p.dt_diagnostics;
        h->time_prog = time;
        ha[i].ctl = h->ctl;
        ha[i].tf = time;
        ha[i].bsl = bsl[i].bsl_now;
        ha[i].A_ocean = bsl[i].A_ocean_now;
        ha[i].method = bsl[i].method;
        ha[i].write_bsl = (bsl[i].method == 0 || bsl[i].method == 1) ? 1 : 0;
    }
    if (cudaMemcpyAsync(b->dargs[b->ring], ha, b->nm * sizeof(BArgs), cudaMemcpyHostToDevice, b->s) != cudaSuccess)
        return FI_E_CUDA;
    batch_set_args(b->dargs[b->ring], b->nm, b->s);
    if (cudaEventRecord(b->args_ev[b->ring], b->s) != cudaSuccess) return FI_E_CUDA;
    b->ring = (b->ring + 1) % fi_batch::kRing;
    if (b->eager) return b->mixed ? batch_eager<float>(b, diag) : batch_eager<double>(b, diag);
    if (!b->g[key]) {
        cudaGraph_t graph = nullptr;
        const int rc = b->mixed ? batch_capture<float>(b, diag, &graph) : batch_capture<double>(b, diag, &graph);
        if (rc) return rc;
        const cudaError_t e = cudaGraphInstantiate(&b->g[key], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return FI_E_CUDA;
    }
    if (cudaGraphLaunch(b->g[key], b->s) != cudaSuccess) return FI_E_CUDA;
    return FI_OK;
}

int fi_batch_wait(fi_batch* b, int32_t* status)
{
    if (!b) return FI_E_ARG;
    if (cudaStreamSynchronize(b->s) != cudaSuccess) return FI_E_CUDA;
    int first = FI_OK;
    for (int i = 0; i < b->nm; ++i) {
        const int rc = fi_synchronize(b->hs[i]);
        if (status) status[i] = rc;
        if (rc && first == FI_OK) first = rc;
    }
    return first;
}

int fi_batch_destroy(fi_batch* b)
{
    if (!b) return FI_E_ARG;
    batch_free(b);
    return FI_OK;
}
