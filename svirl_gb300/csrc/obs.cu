// Observables of one GL instance: free energy (one launch, FP64 accumulation,
// deterministic last-CTA finish), magnetic field, total current and supercurrent
// densities, and the plaquette-winding vortex candidate scan.
//
// Reference: svirl/cuda/observables.h:4-362, svirl/observables/observables.py:29-149,
// svirl/observables/vortex_detector.py:31-72.
#include <mutex>
#include <string>

#include "glgpu_internal.h"
#include "glgpu_phys.cuh"

namespace glgpu {

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_energy(Geo g, double kappa2, double eps0, const T* eps_sp, double H, const uint8_t* mt,
         const C2<T>* __restrict__ psi, const T* abei, const T* ab, double* partials, unsigned* counter, double* out) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    T v[1] = {T(0)};
    if (n < g.N) v[0] = energy_density<T>(g, (T)kappa2, (T)eps0, eps_sp, (T)H, mt, psi, abei, ab, PhaseLinks<T>{abei, ab}, n);
    grid_sum_finish(v, partials, counter, out, g.dxdy);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_magnetic_field(Geo g, const T* abei, const T* ab, T* B) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    if (n >= g.Nxc * g.Nyc) return;
    const int i = n % g.Nxc, j = n / g.Nxc;
    const T idx = GT(g, idx), idy = GT(g, idy);
    T b = T(0);
    if (abei) b += cell_curl(g, abei, i, j, idx, idy);
    if (ab) b += cell_curl(g, ab, i, j, idx, idy);
    B[n] = b;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_current_density(Geo g, double kappa2, double H, const T* abei, const T* ab, T* out) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    if (n >= g.N) return;
    const int i = n % g.Nx, j = n / g.Nx;
    if (i < g.Nx - 1) out[i + (g.Nx - 1) * j] = (T)kappa2 * curlcurl_link<T>(g, abei, ab, (T)H, i, j, true);
    if (j < g.Ny - 1) out[g.Na + i + g.Nx * j] = (T)kappa2 * curlcurl_link<T>(g, abei, ab, (T)H, i, j, false);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_supercurrent_density(Geo g, const uint8_t* mt, const C2<T>* __restrict__ psi, const T* abei, const T* ab, T* out) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    if (n >= g.N) return;
    const int i = n % g.Nx, j = n / g.Nx;
    const unsigned cb = cell_bits(g, mt, i, j);
    const C2<T> p0 = psi[n];
    if (i < g.Nx - 1) {
        const int na = i + (g.Nx - 1) * j;
        T jl = T(0);
        if (GL_PM(cb) || GL_PP(cb)) {
            const T r = T(0.5) * ((GL_PM(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
            jl = r * GT(g, idx) * js_of<T>(p0, GT(g, dx) * link_phase(abei, ab, na), psi[n + 1]);
        }
        out[na] = jl;
    }
    if (j < g.Ny - 1) {
        const int nb = g.Na + i + g.Nx * j;
        T jl = T(0);
        if (GL_MP(cb) || GL_PP(cb)) {
            const T r = T(0.5) * ((GL_MP(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
            jl = r * GT(g, idy) * js_of<T>(p0, GT(g, dy) * link_phase(abei, ab, nb), psi[n + g.Nx]);
        }
        out[nb] = jl;
    }
}

// Plaquette winding per cell in FP64 (svirl/observables/vortex_detector.py:55-72)
// with a relaxed predicate (|v| > 0.45 and |v - round(v)| < 0.15), so the exact
// predicate, applied afterwards to the copied corner data, selects a subset.
__device__ __forceinline__ double pmod(double x, double m) { return x - floor(x / m) * m; }

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_vortex_scan(Geo g, double H, const C2<T>* __restrict__ psi, const T* __restrict__ ab, int cap,
              int* count, int* cells, T* corners) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    if (n >= g.Nxc * g.Nyc) return;
    const int i = n % g.Nxc, j = n / g.Nxc;
    const int Nxa = g.Nx - 1;
    const C2<T> p00 = psi[i + g.Nx * j], pp0 = psi[i + 1 + g.Nx * j];
    const C2<T> ppp = psi[i + 1 + g.Nx * (j + 1)], p0p = psi[i + g.Nx * (j + 1)];
    const T a00 = ab[i + Nxa * j], a0p = ab[i + Nxa * (j + 1)];
    const T b00 = ab[g.Na + i + g.Nx * j], bp0 = ab[g.Na + i + 1 + g.Nx * j];
    const double t00 = atan2((double)p00.y, (double)p00.x), tp0 = atan2((double)pp0.y, (double)pp0.x);
    const double tpp = atan2((double)ppp.y, (double)ppp.x), t0p = atan2((double)p0p.y, (double)p0p.x);
    const double pi = 3.141592653589793, tp = 2.0 * pi;
    const double v = -(0.5 / pi) * (pmod(tp0 - t00 - g.dx * (double)a00 + pi, tp) + pmod(tpp - tp0 - g.dy * (double)bp0 + pi, tp)
                                    + pmod(t0p - tpp + g.dx * (double)a0p + pi, tp) + pmod(t00 - t0p + g.dy * (double)b00 + pi, tp)
                                    - 4.0 * pi + g.dx * g.dy * H);
    if (fabs(v) > 0.45 && fabs(v - rint(v)) < 0.15) {
        int k = atomicAdd(count, 1);
        if (k < cap) {
            cells[k] = n;
            T* c = corners + (size_t)k * 12;
            c[0] = p00.x; c[1] = p00.y; c[2] = pp0.x; c[3] = pp0.y;
            c[4] = ppp.x; c[5] = ppp.y; c[6] = p0p.x; c[7] = p0p.y;
            c[8] = a00; c[9] = a0p; c[10] = b00; c[11] = bp0;
        }
    }
}

// Grid-stride FP64 sum of n vectors of NV doubles.
template <int NV>
__global__ void __launch_bounds__(kThreads)
k_vsum(const double* __restrict__ x, long long n, double* partials, unsigned* counter, double* out) {
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    for (long long m = (long long)blockIdx.x * kThreads + threadIdx.x; m < n; m += (long long)gridDim.x * kThreads)
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] += x[m * NV + k];
    grid_sum_finish(v, partials, counter, out, 1.0);
}

// ---------------------------------------------------------------------------
// host entry points
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// Free energy with no allocation by the library (glgpu_free_energy_noalloc).
//
// For callers that cannot let a library call cudaMalloc: a host process whose
// own allocator owns the device memory (a framework's caching allocator, a
// pre-sized arena under a fixed memory budget), or a plugin that must not
// allocate behind its host's back.  The caller passes the state and the output
// as device pointers; the reduction's scratch (one partial sum per CTA and the
// last-CTA ticket counter) lives in the static array below, which every GPU that
// loads libglgpu.so holds until the process exits: 32769 doubles = 256 KB + 8 B.
// Grids up to kNoAllocMaxNodes nodes fit; larger grids are rejected.
// ---------------------------------------------------------------------------
constexpr long long kNoAllocMaxNodes = 1LL << 23;                       // 8,388,608 nodes
constexpr int kNoAllocMaxBlocks = (int)(kNoAllocMaxNodes / kThreads);   // 32,768 CTAs
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks + 1];  // partials, then the counter

// Device address of g_noalloc_scratch for each device (host code cannot use the
// symbol itself: on the host it names a stand-in, not device memory).  Looked up
// again on every call that is not being captured into a graph, so that a device
// reset (which reloads the module at another address) leaves no stale pointer;
// a call under stream capture uses the address of the last call outside capture.
static std::mutex g_noalloc_mutex;
static double* g_noalloc_addr[256] = {nullptr};

static double* noalloc_scratch(int dev, cudaStream_t stream, std::string* why) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (dev < 0 || dev >= 256) {
        *why = "device ordinal out of range";
        return nullptr;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cs);
    if (e != cudaSuccess) {
        *why = std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e);
        return nullptr;
    }
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            *why = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return nullptr;
        }
        g_noalloc_addr[dev] = (double*)p;
    } else if (!g_noalloc_addr[dev]) {
        *why = "the first call on a device must come before any stream capture";
        return nullptr;
    }
    return g_noalloc_addr[dev];
}

int free_energy_noalloc(const glgpu_grid* grid, const glgpu_params* p, const void* psi, const void* ab,
                        const void* abei, const uint8_t* mt, double* energy, cudaStream_t stream) {
    if (!grid || !p || !psi || !energy) return set_error(nullptr, GLGPU_E_ARG, "glgpu_free_energy_noalloc: NULL argument");
    if (grid->Nx < 4 || grid->Ny < 4 || (grid->dtype != 4 && grid->dtype != 8) || !(grid->dx > 0.0) || !(grid->dy > 0.0))
        return set_error(nullptr, GLGPU_E_ARG, "glgpu_free_energy_noalloc: bad grid (Nx, Ny >= 4, dtype 4 or 8, dx, dy > 0)");
    const long long n = (long long)grid->Nx * grid->Ny;
    if (n > kNoAllocMaxNodes)
        return set_error(nullptr, GLGPU_E_ARG,
                         "glgpu_free_energy_noalloc: " + std::to_string(n) + " nodes exceed the static scratch's maximum of " +
                             std::to_string(kNoAllocMaxNodes) + " nodes; use glgpu_free_energy on a handle");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(nullptr, GLGPU_E_CUDA, std::string("glgpu_free_energy_noalloc: ") + cudaGetErrorString(e));
    std::string why;
    double* scratch = noalloc_scratch(dev, stream, &why);
    if (!scratch) return set_error(nullptr, GLGPU_E_CUDA, "glgpu_free_energy_noalloc: " + why);
    unsigned* counter = (unsigned*)(scratch + kNoAllocMaxBlocks);
    const Geo g = make_geo(grid->Nx, grid->Ny, grid->dx, grid->dy);
    const bool finite = p->kappa > 0.0 && !std::isinf(p->kappa);
    const double k2 = finite ? p->kappa * p->kappa : -1.0;
    // the ticket counter must start at zero; the last call may have been interrupted
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), stream);
    if (e == cudaSuccess) {
        const int nb = blocks_for(n);
        if (grid->dtype == 8)
            k_energy<double><<<nb, kThreads, 0, stream>>>(g, k2, p->epsilon, nullptr, p->H, mt, (const double2*)psi,
                                                         (const double*)abei, (const double*)ab, scratch, counter, energy);
        else
            k_energy<float><<<nb, kThreads, 0, stream>>>(g, k2, p->epsilon, nullptr, p->H, mt, (const float2*)psi,
                                                        (const float*)abei, (const float*)ab, scratch, counter, energy);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return set_error(nullptr, GLGPU_E_CUDA, std::string("glgpu_free_energy_noalloc: ") + cudaGetErrorString(e));
    return GLGPU_OK;
}

int reduce_sum(glgpu_handle* h, const double* x, long long n, int nv, double* out) {
    if (!x || !out || n < 0 || !(nv == 1 || nv == 5 || nv == 17)) return set_error(h, GLGPU_E_ARG, "reduce_sum: bad arguments");
    double* dx = nullptr;
    const size_t bytes = (size_t)(n > 0 ? n : 1) * nv * sizeof(double);
    if (cudaMalloc(&dx, bytes) != cudaSuccess) return set_error(h, GLGPU_E_OOM, "reduce_sum: out of device memory");
    cudaError_t e = n > 0 ? cudaMemcpyAsync(dx, x, (size_t)n * nv * sizeof(double), cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
    long long nb = (n + kThreads - 1) / kThreads;
    int grid = (int)(nb < 1 ? 1 : (nb > h->ntiles ? h->ntiles : nb));
    if (e == cudaSuccess) {
        if (nv == 1) k_vsum<1><<<grid, kThreads, 0, h->stream>>>(dx, n, h->partials, h->counter, h->dscal + 0);
        else if (nv == 5) k_vsum<5><<<grid, kThreads, 0, h->stream>>>(dx, n, h->partials, h->counter, h->dscal + 0);
        else k_vsum<17><<<grid, kThreads, 0, h->stream>>>(dx, n, h->partials, h->counter, h->dscal + 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->hscal, h->dscal, nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dx);
    if (e != cudaSuccess) return cuda_check(h, e, "reduce_sum");
    for (int k = 0; k < nv; ++k) out[k] = h->hscal[k];
    return GLGPU_OK;
}

static inline bool finite_kappa(const glgpu_handle* h) { return h->p.kappa > 0.0 && !std::isinf(h->p.kappa); }
static inline double kappa2_of(const glgpu_handle* h) { return finite_kappa(h) ? h->p.kappa * h->p.kappa : -1.0; }

int obs_free_energy_device(glgpu_handle* h) {
    const int nb = blocks_for(h->g.N);
    if (h->dtype == 8)
        k_energy<double><<<nb, kThreads, 0, h->stream>>>(h->g, kappa2_of(h), h->p.epsilon, (const double*)h->eps_sp, h->p.H, h->mt,
                                                        (const double2*)h->psi[0], (const double*)h->abei, (const double*)h->ab[0],
                                                        h->partials, h->counter, h->dscal + 20);
    else
        k_energy<float><<<nb, kThreads, 0, h->stream>>>(h->g, kappa2_of(h), h->p.epsilon, (const float*)h->eps_sp, h->p.H, h->mt,
                                                       (const float2*)h->psi[0], (const float*)h->abei, (const float*)h->ab[0],
                                                       h->partials, h->counter, h->dscal + 20);
    return cuda_check(h, cudaGetLastError(), "free_energy launch");
}

int obs_free_energy(glgpu_handle* h, double* out) {
    int rc = obs_free_energy_device(h);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(h->hscal + 20, h->dscal + 20, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "free_energy");
    *out = h->hscal[20];
    return GLGPU_OK;
}

static int copy_out(glgpu_handle* h, void* host, size_t bytes, const char* what) {
    cudaError_t e = cudaMemcpyAsync(host, h->out, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, what);
}

int obs_magnetic_field(glgpu_handle* h, void* host_out) {
    const int nc = h->g.Nxc * h->g.Nyc;
    if (h->dtype == 8)
        k_magnetic_field<double><<<blocks_for(nc), kThreads, 0, h->stream>>>(h->g, (const double*)h->abei, (const double*)h->ab[0], (double*)h->out);
    else
        k_magnetic_field<float><<<blocks_for(nc), kThreads, 0, h->stream>>>(h->g, (const float*)h->abei, (const float*)h->ab[0], (float*)h->out);
    return copy_out(h, host_out, (size_t)nc * real_size(h), "magnetic_field");
}

int obs_supercurrent_density(glgpu_handle* h, void* host_out) {
    if (h->dtype == 8)
        k_supercurrent_density<double><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, h->mt, (const double2*)h->psi[0],
                                                                                      (const double*)h->abei, (const double*)h->ab[0], (double*)h->out);
    else
        k_supercurrent_density<float><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, h->mt, (const float2*)h->psi[0],
                                                                                     (const float*)h->abei, (const float*)h->ab[0], (float*)h->out);
    return copy_out(h, host_out, (size_t)h->g.Nab * real_size(h), "supercurrent_density");
}

int obs_current_density(glgpu_handle* h, void* host_out) {
    if (!finite_kappa(h)) return obs_supercurrent_density(h, host_out);  // observables.py:89-90
    if (h->dtype == 8)
        k_current_density<double><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, kappa2_of(h), h->p.H, (const double*)h->abei,
                                                                                 (const double*)h->ab[0], (double*)h->out);
    else
        k_current_density<float><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, kappa2_of(h), h->p.H, (const float*)h->abei,
                                                                                (const float*)h->ab[0], (float*)h->out);
    return copy_out(h, host_out, (size_t)h->g.Nab * real_size(h), "current_density");
}

int obs_vortex_candidates(glgpu_handle* h, int cap, int* n_out, int32_t* cells, void* corners) {
    if (cap < 0 || !n_out) return set_error(h, GLGPU_E_ARG, "vortex_candidates: bad arguments");
    if (cap > h->vort_cap) {
        if (h->vort) cudaFree(h->vort);
        h->vort = nullptr;
        h->vort_cap = 0;
        size_t bytes = (size_t)cap * (sizeof(int) + 12 * real_size(h));
        if (cudaMalloc(&h->vort, bytes) != cudaSuccess) return set_error(h, GLGPU_E_OOM, "vortex_candidates: out of memory");
        h->vort_cap = cap;
    }
    cudaError_t e = cudaMemsetAsync(h->vort_n, 0, sizeof(int), h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "vortex_candidates");
    const int nc = h->g.Nxc * h->g.Nyc;
    int* dcells = (int*)h->vort;
    void* dcorn = (char*)h->vort + (size_t)h->vort_cap * sizeof(int);
    if (h->dtype == 8)
        k_vortex_scan<double><<<blocks_for(nc), kThreads, 0, h->stream>>>(h->g, h->p.H, (const double2*)h->psi[0], (const double*)h->ab[0],
                                                                         cap, h->vort_n, dcells, (double*)dcorn);
    else
        k_vortex_scan<float><<<blocks_for(nc), kThreads, 0, h->stream>>>(h->g, h->p.H, (const float2*)h->psi[0], (const float*)h->ab[0],
                                                                        cap, h->vort_n, dcells, (float*)dcorn);
    int cnt = 0;
    e = cudaMemcpyAsync(&cnt, h->vort_n, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "vortex_candidates");
    *n_out = cnt;
    const int m = cnt < cap ? cnt : cap;
    if (m > 0) {
        if (cells) e = cudaMemcpyAsync(cells, dcells, (size_t)m * sizeof(int), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess && corners)
            e = cudaMemcpyAsync(corners, dcorn, (size_t)m * 12 * real_size(h), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return cuda_check(h, e, "vortex_candidates copy");
    }
    return GLGPU_OK;
}

}  // namespace glgpu
