// me_noalloc.cu -- full-search motion estimation that allocates nothing.
//
// Some callers cannot call cudaMalloc once they are running: real-time
// encoders that fix their device memory budget at start-up, plugins hosted
// by an application or framework that owns every device allocation, and
// code paths whose rules forbid allocator calls after initialisation.  For
// them, vppgpu_me_full_estimate_noalloc runs the same kernels as
// vppgpu_me_estimate_device, but every intermediate buffer (packed source,
// padded reference, block energies, per-macroblock results, SSD tables of
// tie macroblocks, control words) lives
// in one file-scope device array of fixed size, g_noalloc_scratch below.
// The caller passes device inputs and outputs; the call makes no
// cudaMalloc, cudaFree or other allocating call.
//
// Limits: at most VPPGPU_NOALLOC_MAX_MBS (396) stored macroblocks, e.g. CIF
// 352x288, width and height at most VPPGPU_NOALLOC_MAX_DIM (1024); larger
// frames are rejected with VPPGPU_ERR_UNSUPPORTED.  The array takes 12 MiB on
// every GPU that loads the library, for as long as the process runs.
//
// Sharing: all calls use the same array and it keeps the previous call's
// contents.  The words that must start at zero -- the status, counters and
// the dirty bitmap (MeCtrl and changed[0 .. sweep_limit)) -- are cleared by
// every call; everything else is written before it is read.  Calls that
// overlap on the GPU (other host threads, or other streams) race on the array
// and must be serialised by the caller.
//
// Set-up: the first call on a device, made with that device current, looks
// up the array's device address with cudaGetSymbolAddress and configures the
// kernels.  With CUDA's lazy module loading (the default) that first call is
// also when the driver reserves the array, so a caller with a fixed budget
// makes it at start-up; make it before any stream capture begins.  Every call
// is synchronous: it returns once the results are written.
#include <mutex>

#include "me_full_common.cuh"

namespace {

constexpr size_t kSrcBytes = 131072;                       // packed source, W*H bytes
constexpr size_t kRefBytes = 327680;                       // padded reference, (W+96)*(H+96) bytes
constexpr size_t kSpecBytes = 8192;                        // 5 ints per macroblock
constexpr size_t kStateBytes = 4864;                       // 3 ints per macroblock
constexpr size_t kCtrlBytes = 256;                         // vppgpu::MeCtrl
constexpr size_t kChangedBytes = 1792;                     // sweep counters + dirty bitmap
constexpr size_t kCacheBytes = 202752;                     // KCACHE 16-byte records per macroblock
constexpr size_t kDictBytes = 256;                         // NDICT vectors
constexpr size_t kHpelBytes = 3 * kRefBytes;               // b, h, j planes of the padded reference
// Wavefront records, wave_rec_count(cols, rows): at most 2*(12+62)*32 = 4736
// for 396 macroblocks no wider or taller than 64 (rows 33..64 leave at most
// 12 columns; 32 rows or fewer at most 64 columns, 4032).
constexpr size_t kWaveRecBytes = 4736 * sizeof(vppgpu::WaveRec);
constexpr size_t kChoiceBytes = 1600;                      // one int per macroblock
constexpr size_t kTieListBytes = 1600;                     // one int per macroblock
constexpr size_t kJobBytes = 64;                           // vppgpu::JobDesc
constexpr size_t kTableBytes = (size_t)VPPGPU_NOALLOC_MAX_MBS * 64 * 64 * 4;
constexpr size_t kEnergyBytes = 4 * kRefBytes;               // one int per padded reference sample
constexpr size_t kOffSrc = 0;
constexpr size_t kOffRef = kOffSrc + kSrcBytes;
constexpr size_t kOffSpec = kOffRef + kRefBytes;
constexpr size_t kOffState = kOffSpec + kSpecBytes;
constexpr size_t kOffCtrl = kOffState + kStateBytes;
constexpr size_t kOffChanged = kOffCtrl + kCtrlBytes;
constexpr size_t kOffCache = kOffChanged + kChangedBytes;
constexpr size_t kOffDict = kOffCache + kCacheBytes;
constexpr size_t kOffHpel = kOffDict + kDictBytes;
constexpr size_t kOffWaveRec = kOffHpel + kHpelBytes;
constexpr size_t kOffChoice = kOffWaveRec + kWaveRecBytes;
constexpr size_t kOffTieList = kOffChoice + kChoiceBytes;
constexpr size_t kOffJob = kOffTieList + kTieListBytes;
constexpr size_t kOffTables = kOffJob + kJobBytes;
constexpr size_t kOffEnergy = kOffTables + kTableBytes;
static_assert(sizeof(vppgpu::JobDesc) <= kJobBytes && kOffJob % 16 == 0, "job descriptor does not fit");
static_assert(16 * vppgpu::KCACHE * VPPGPU_NOALLOC_MAX_MBS <= kCacheBytes && 4 * vppgpu::NDICT <= kDictBytes,
              "resolve caches do not fit");
static_assert(sizeof(vppgpu::WaveRec) * VPPGPU_NOALLOC_MAX_MBS <= kWaveRecBytes &&
                  4 * VPPGPU_NOALLOC_MAX_MBS <= kChoiceBytes,
              "wavefront records do not fit");
static_assert(kOffSpec % 16 == 0 && kOffCache % 16 == 0 && kOffHpel % 16 == 0 &&
                  kOffWaveRec % 16 == 0 && kOffTables % 16 == 0 && kOffEnergy % 16 == 0,
              "vector records and planes need 16-byte alignment");
constexpr size_t kScratchBytes = 12u << 20;
static_assert(kOffEnergy + kEnergyBytes <= kScratchBytes, "scratch layout exceeds the array");
static_assert(sizeof(vppgpu::MeCtrl) <= kCtrlBytes, "control block does not fit");
static_assert(5 * 4 * VPPGPU_NOALLOC_MAX_MBS <= kSpecBytes && 3 * 4 * VPPGPU_NOALLOC_MAX_MBS <= kStateBytes &&
                  4 * (vppgpu::RELAX_SWEEPS + 2 + (VPPGPU_NOALLOC_MAX_MBS + 31) / 32) <= kChangedBytes,
              "per-macroblock arrays do not fit");

// The only device memory this entry point uses.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
    bool ready;
    unsigned char* scratch;  // device address of g_noalloc_scratch on this device
    int sm_count;
    int resolve_cap;         // co-resident blocks of the cooperative resolve kernel
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mutex;

int setup_device(int dev, DeviceSetup** out)
{
    if (dev < 0 || dev >= kMaxDevices) return VPPGPU_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup& s = g_setup[dev];
    if (!s.ready) {
        int major = 0, minor = 0, sms = 0;
        VPP_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
        VPP_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
        VPP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (major != 10 || minor != 3) return VPPGPU_ERR_NO_DEVICE;
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return vppgpu::cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
        vppgpu_ctx probe = {};
        probe.device = dev;
        probe.sm_count = sms;
        int cap = 0;
        int rc = vppgpu::full_prepare(&probe, 1 << 28, &cap);
        if (rc) return rc;
        s.scratch = (unsigned char*)p;
        s.sm_count = sms;
        s.resolve_cap = cap;
        s.ready = true;
    }
    *out = &s;
    return VPPGPU_OK;
}

}  // namespace

extern "C" int vppgpu_me_full_estimate_noalloc(const short* d_src, const short* d_ref, int width, int height,
                                               int motion_range, const unsigned char* d_dist_included,
                                               const int* d_mb_slice, short* d_mv_out, int* d_mb_dist_out,
                                               long* avg_distortion, void* cuda_stream)
{
    if (!d_src || !d_ref || !d_mv_out) return VPPGPU_ERR_INVALID_ARG;
    if (((uintptr_t)d_src | (uintptr_t)d_ref | (uintptr_t)d_mv_out) & 3) return VPPGPU_ERR_INVALID_ARG;
    if (width < 16 || height < 16 || (width % 16) != 0 || motion_range < 4) return VPPGPU_ERR_INVALID_ARG;
    const int cols = width / 16, nmb = cols * (height / 16);
    if (width > VPPGPU_NOALLOC_MAX_DIM || height > VPPGPU_NOALLOC_MAX_DIM || nmb > VPPGPU_NOALLOC_MAX_MBS ||
        motion_range > 128 || (size_t)width * height > kSrcBytes ||
        (size_t)(width + 2 * vppgpu::PAD) * (height + 2 * vppgpu::PAD) > kRefBytes ||
        vppgpu::wave_rec_count(cols, height / 16) * sizeof(vppgpu::WaveRec) > kWaveRecBytes)
        return VPPGPU_ERR_UNSUPPORTED;

    int dev = 0;
    VPP_CUDA(cudaGetDevice(&dev));
    DeviceSetup* s = nullptr;
    int rc = setup_device(dev, &s);
    if (rc) return rc;

    // a context on the stack: the caller's stream, no owned resources
    vppgpu_ctx ctx = {};
    ctx.device = dev;
    ctx.sm_count = s->sm_count;
    ctx.stream = (cudaStream_t)cuda_stream;

    unsigned char* base = s->scratch;
    vppgpu::FullArgs a{};
    a.W = width;
    a.H = height;
    a.cols = cols;
    a.nmb = nmb;
    a.motion_range = motion_range;
    a.rstride = width + 2 * vppgpu::PAD;
    a.src8 = base + kOffSrc;
    a.refp = base + kOffRef;
    a.hpel = base + kOffHpel;
    a.plane_size = (size_t)a.rstride * (height + 2 * vppgpu::PAD);
    a.wave_rec = (vppgpu::WaveRec*)(base + kOffWaveRec);
    a.wave_choice = (int*)(base + kOffChoice);
    a.tie_list = (int*)(base + kOffTieList);
    int* spec = (int*)(base + kOffSpec);
    a.spec4 = reinterpret_cast<int4*>(spec);
    a.spec_imv = spec + 4 * nmb;
    a.tables = (int*)(base + kOffTables);
    a.energy = (const int*)(base + kOffEnergy);
    a.cache = (int4*)(base + kOffCache);
    a.dict = (int*)(base + kOffDict);
    int* state = (int*)(base + kOffState);
    a.final_mv = state;
    a.final_dist = state + nmb;
    a.pred_used = state + 2 * nmb;
    a.job = (const vppgpu::JobDesc*)(base + kOffJob);
    a.ctrl = (vppgpu::MeCtrl*)(base + kOffCtrl);
    a.changed = (int*)(base + kOffChanged);
    a.lambda = 1.05;
    a.sweep_limit = vppgpu::RELAX_SWEEPS + 2 + (nmb + 31) / 32;  // sweep counters, then the dirty bitmap
    a.dirty = reinterpret_cast<unsigned*>(a.changed + vppgpu::RELAX_SWEEPS + 2);
    a.relax_sweeps = 8;
    a.grid_sweeps = 8;
    a.relax_blocks_per_sm = 4;
    a.mrc = nullptr;
    a.lattice = nullptr;
    a.search_cache = nullptr;
    a.tie_runs = nullptr;
    a.spin_limit = 20000000LL;

    // the words that must start at zero on every call
    VPP_CUDA(cudaMemsetAsync(a.ctrl, 0, sizeof(vppgpu::MeCtrl), ctx.stream));
    VPP_CUDA(cudaMemsetAsync(a.changed, 0, sizeof(int) * (size_t)a.sweep_limit, ctx.stream));
    int grid = (nmb + 7) / 8;
    if (grid > s->resolve_cap) grid = s->resolve_cap;
    rc = vppgpu::set_job(&ctx, (vppgpu::JobDesc*)(base + kOffJob),
                         vppgpu::JobDesc{d_src, d_ref, d_dist_included, d_mb_slice, (int*)d_mv_out, d_mb_dist_out, nullptr});
    if (rc) return rc;
    vppgpu::SearchMaps maps;  // host-side descriptors of the array's planes, passed by value
    if ((rc = vppgpu::search_maps_encode(a, &maps))) return rc;
    rc = vppgpu::full_launch(&ctx, a, maps, nmb, grid, nullptr);
    if (rc) return rc;

    vppgpu::MeCtrl h = {};
    VPP_CUDA(cudaMemcpyAsync(&h, a.ctrl, sizeof(h), cudaMemcpyDeviceToHost, ctx.stream));
    VPP_CUDA(cudaStreamSynchronize(ctx.stream));
    if (h.status & vppgpu::ST_PIXEL_RANGE) return VPPGPU_ERR_PIXEL_RANGE;
    if (h.status & vppgpu::ST_TIMEOUT) return VPPGPU_ERR_TIMEOUT;
    if (avg_distortion) *avg_distortion = h.count ? (long)(h.total / h.count) : 0;
    return VPPGPU_OK;
}
