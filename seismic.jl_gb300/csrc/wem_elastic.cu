// wem_elastic.cu -- elastic shot-profile migration and its forward operator on the GPU:
// the reference's ewem / elastic_extrap1f / elastic_separate_3d (src/Imaging/c/ewem.c:3-741),
// 2-D grids (nmy = 1) here; 3-D grids (nmy > 1) go to wem_elastic3d.cu.
//
// Everything that depends only on (frequency, depth) -- the phase rows of the P and S layer
// slownesses, the slowness corrections and the separation coefficients of every wavenumber -- is
// built once per frequency band by wem_ewem_tables_kernel, one record per (frequency, depth),
// and shared by every shot. The depth kernel carries several shots of one frequency per CTA,
// each as a receiver pair of row teams (N/16 threads each, a row of N samples in registers as in
// the acoustic depth kernels): the components (ux, uz), separated at every depth into the P and
// S2 potentials (elastic_separate_3d), continued with the split-step operator of their own
// velocity (ssop with vp or vs), and recombined into components. A pair meets in two shared
// spectrum buffers for the separation and the recombination, which mix its two rows at each
// wavenumber. One source team advances the group's source rows. Migration (adj): the sources go
// down beside the receivers and each depth adds Re(conj(smig) P) into the P image and
// Re(conj(smig) S2) into the S image (compensated accumulators per CTA and shot slot, reduced in
// a fixed order). Modelling: the source pass stores smig for every depth, then the receivers go
// up with smig * image injected into P and S2. The y component and the S1 image stay zero, as
// in the reference (its S1 separation is commented out, ewem.c:579-587).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/shotwem_gb300.h"
#include "wem_elastic.cuh"

namespace gbwem {
int set_error(int code, const char *msg);  // wem_api.cu: records wem_last_error()
// wem_elastic3d.cu: the same operator on 3-D grids (nmy > 1)
int wem_elastic3d(int device, const wem_params &p, const float *vp, const float *vs, const float *wav, int nshot,
                  const float *sx, const float *sy, float *ux, float *uz, float *mpp, float *mps2, int adj, float *ms);
}
void bluestein_tables(int L, int N, float2 *chirp, float2 *gq);  // wem_api.cu
int row_length_2d(int nkx, bool *blu);                           // wem_api.cu

using namespace gbwem;

namespace gbwem {
// The tables of one (frequency, depth) record per block: the phase entries and the slowness
// corrections of the P and S layers, and the separation coefficients of elastic_separate_3d
// (ewem.c:598-611) at every wavenumber; the float operations of the in-kernel forms they
// replace (bit-identical), shared by every shot of the frequency.
__global__ void __launch_bounds__(256) wem_ewem_tables_kernel(const EwemArgs a)
{
    const MigArgs &m = a.m;
    const int rec = blockIdx.x, iz = rec % m.nz, iwc = rec / m.nz;
    const int L = a.nkx, nmx = m.nmx;
    const EwemRec R(L, nmx);
    float *out = a.tabs + (size_t)rec * R.floats();
    float2 *php = reinterpret_cast<float2 *>(out + R.php()), *phs = reinterpret_cast<float2 *>(out + R.phs());
    float2 *cp = reinterpret_cast<float2 *>(out + R.cp()), *cs = reinterpret_cast<float2 *>(out + R.cs());
    float *sep = out + R.sep();
    const int iw = m.ifmin + a.wbase + iwc;
    const float w = __fmul_rn((float)iw, m.dw);
    const float w2 = __fmul_rn(w, w);
    const float pp = a.po_p[iz], ps = a.po_s[iz];
    const float sp2 = __fmul_rn(pp, pp), ss2 = __fmul_rn(ps, ps);
    for (int k = threadIdx.x; k < R.rh; k += blockDim.x) {
        const float kx = __fmul_rn(m.dkx, (float)k);
        php[k] = k < L / 2 + 1 ? phase_entry(w2, sp2, kx, m.dz, m.inv_n) : make_float2(0.f, 0.f);
        phs[k] = k < L / 2 + 1 ? phase_entry(w2, ss2, kx, m.dz, m.inv_n) : make_float2(0.f, 0.f);
    }
    const float *dp = a.pd_p + (size_t)iz * nmx, *ds = a.pd_s + (size_t)iz * nmx;
    for (int x = threadIdx.x; x < R.nmxp; x += blockDim.x) {
        float sn = 0.f, c = 0.f;
        if (x < nmx) sincosf(__fmul_rn(__fmul_rn(w, dp[x]), m.dz), &sn, &c);
        cp[x] = make_float2(c, sn);
        sn = c = 0.f;
        if (x < nmx) sincosf(__fmul_rn(__fmul_rn(w, ds[x]), m.dz), &sn, &c);
        cs[x] = make_float2(c, sn);
    }
    const float vp = a.vp_mean[iz], vs = a.vs_mean[iz];
    for (int k = threadIdx.x; k < R.lp; k += blockDim.x) {
        SepCoef c{};
        if (k < L) c = sep_coef(kx_signed(k, L, m.dkx), w, vp, vs);
        sep[k] = c.kxp;
        sep[R.lp + k] = c.kzp;
        sep[2 * R.lp + k] = c.kxs;
        sep[3 * R.lp + k] = c.kzs;
        sep[4 * R.lp + k] = c.norm;
    }
}
}  // namespace gbwem

// ------------------------------------------------------------------ host side
namespace {

int ewem_launch(int nfft, int blu, int adj, const EwemArgs *a, int nsm, int nitems, cudaStream_t st, int *grid,
                size_t *smem)
{
    switch (nfft) {
    case 64: return ewem_launch_n<64>(blu, adj, a, nsm, nitems, st, grid, smem);
    case 128: return ewem_launch_n<128>(blu, adj, a, nsm, nitems, st, grid, smem);
    case 256: return ewem_launch_n<256>(blu, adj, a, nsm, nitems, st, grid, smem);
    case 512: return ewem_launch_n<512>(blu, adj, a, nsm, nitems, st, grid, smem);
    case 1024: return ewem_launch_n<1024>(blu, adj, a, nsm, nitems, st, grid, smem);
    case 2048: return ewem_launch_n<2048>(blu, adj, a, nsm, nitems, st, grid, smem);
    default: return -2;
    }
}

// device buffers of one call, freed on every return
struct Bufs {
    std::vector<void *> ptrs;
    ~Bufs()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T> T *get(size_t n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
};

thread_local float g_last_ms = 0.f;  // per calling thread

}  // namespace

#define ECK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return set_error(WEM_ERR_CUDA, cudaGetErrorString(e_));                   \
    } while (0)

extern "C" WEM_API int wem_elastic(int device, const wem_params *pp, const float *vp, const float *vs,
                                   const float *wav, int nshot, const float *sx, const float *sy, float *ux, float *uz,
                                   float *mpp, float *mps2, int adj)
{
    if (!pp || !vp || !vs || !wav || !sx || !ux || !uz || !mpp || !mps2 || nshot < 1)
        return set_error(WEM_ERR_ARG, "wem_elastic: null argument or no shot");
    const wem_params p = *pp;
    if (p.nmy > 1) return wem_elastic3d(device, p, vp, vs, wav, nshot, sx, sy, ux, uz, mpp, mps2, adj, &g_last_ms);
    if (p.nmy != 1) return set_error(WEM_ERR_ARG, "wem_elastic: nmy must be at least 1");
    if (p.nt < 2 || p.nmx < 2 || p.nz < 1 || p.padt < 1 || p.padx < 1 || !(p.dt > 0) || !(p.dmx > 0))
        return set_error(WEM_ERR_ARG, "wem_elastic: invalid grid");
    const int nmx = p.nmx, nz = p.nz, nt = p.nt;
    // grids with ewem.c's own float expressions (ewem.c:44-57)
    const int ntfft = (int)2 * truncf(p.padt * ((float)nt) / 2);
    const int nw = (int)truncf(ntfft / 2) + 1;
    const int nkx = p.padx * nmx;
    const float dkx = 2 * 3.141592653589793 / ((float)nkx) / p.dmx;
    const float dw = 2 * 3.141592653589793 / ((float)ntfft) / p.dt;
    int ifmax, ifmin;
    if (p.fmax * p.dt * ntfft + 1 < nw) ifmax = trunc(p.fmax * p.dt * ntfft) + 1;
    else ifmax = nw;
    if (p.fmin * p.dt * ntfft + 1 < ifmax) ifmin = trunc(p.fmin * p.dt * ntfft);
    else ifmin = 0;
    const int nwf = ifmax - ifmin, nf = (nw - 1) * 2;
    bool blu = false;
    const int nfft = row_length_2d(nkx, &blu);
    if (!nfft || nfft < 64 || nfft > 2048)
        return set_error(WEM_ERR_SIZE, "wem_elastic: padx*nmx must be a power of two in [64, 2048] or another "
                                       "length in [33, 1024]");
    // slowness split of ewem.c:63-82 (float accumulation, double reciprocals)
    std::vector<float> po_p(nz), po_s(nz), pd_p((size_t)nz * nmx), pd_s((size_t)nz * nmx), vpm(nz), vsm(nz);
    for (int iz = 0; iz < nz; iz++) {
        float sp = 0.f, ss = 0.f;
        for (int ix = 0; ix < nmx; ix++) {
            sp += vp[(size_t)ix * nz + iz];
            ss += vs[(size_t)ix * nz + iz];
        }
        sp /= (float)nmx;
        ss /= (float)nmx;
        po_p[iz] = 1. / sp;
        po_s[iz] = 1. / ss;
        for (int ix = 0; ix < nmx; ix++) {
            pd_p[(size_t)iz * nmx + ix] = 1.0 / vp[(size_t)ix * nz + iz] - po_p[iz];
            pd_s[(size_t)iz * nmx + ix] = 1.0 / vs[(size_t)ix * nz + iz] - po_s[iz];
        }
        vpm[iz] = 1. / po_p[iz];
        vsm[iz] = 1. / po_s[iz];
    }
    // boundary_condition (ewem.c:533-551), recomputed per point
    std::vector<float> taper(nmx, 1.f);
    const int lmx = nmx > 100 ? 30 : 0;
    for (int imx = 0; imx < nmx; imx++) {
        if (imx < lmx) taper[imx] = expf(-powf(0.015 * ((float)lmx - imx), 2.));
        if (imx > nmx - lmx) taper[imx] = expf(-powf(0.015 * ((float)imx - nmx + lmx), 2.));
    }
    std::vector<int> igx(nshot);
    for (int s = 0; s < nshot; s++) {
        igx[s] = (int)truncf((sx[s] - p.omx) / p.dmx);  // ewem.c:104
        if (igx[s] < 0 || igx[s] >= nmx) return set_error(WEM_ERR_ARG, "wem_elastic: a source falls outside the grid");
    }
    float max_source = 0.f;
    for (int it = 0; it < nt; it++)
        if (max_source < fabsf(wav[it]) / sqrtf((float)ntfft)) max_source = fabsf(wav[it]) / sqrtf((float)ntfft);
    if (!(max_source > 0.f)) return set_error(WEM_ERR_ARG, "wem_elastic: the wavelet is zero");
    const int ntw = twiddle_table_size(nfft);
    std::vector<float2> tw(ntw + 1);
    twiddle_table_host(nfft, tw.data());
    int chirp_off = 0, bfft_off = 0;
    if (blu) {
        chirp_off = (int)tw.size();
        bfft_off = chirp_off + ((nkx + 1) & ~1);
        tw.resize((size_t)bfft_off + nfft);
        bluestein_tables(nkx, nfft, &tw[chirp_off], &tw[bfft_off]);
    }
    std::vector<float2> wtab(nf);
    for (int k = 0; k < nf; k++) {
        const double an = -6.283185307179586476925286766559 * (double)k / (double)nf;
        wtab[k] = make_float2((float)cos(an), (float)sin(an));
    }
    const float sq = sqrtf((float)ntfft);
    std::vector<float> sc_in(std::max(nwf, 1), 1.f / sq), sc_out(std::max(nwf, 1));
    for (int i = 0; i < nwf; i++) {
        const int iw = ifmin + i;
        sc_out[i] = (iw == 0 || 2 * iw == nf) ? 1.f : 2.f;  // the half-spectrum weights of the c2r (f_op)
    }

    ECK(cudaSetDevice(device));
    int nsm = 0;
    ECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st = nullptr;
    ECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{ st };
    Bufs B;
    const size_t ntr = (size_t)nshot * nmx, nzx = (size_t)nz * nmx;
    float *d_po_p = B.get<float>(nz), *d_po_s = B.get<float>(nz), *d_vpm = B.get<float>(nz), *d_vsm = B.get<float>(nz);
    float *d_pd_p = B.get<float>(nzx), *d_pd_s = B.get<float>(nzx), *d_tap = B.get<float>(nmx);
    float2 *d_tw = B.get<float2>(tw.size()), *d_wtab = B.get<float2>(nf);
    float *d_scin = B.get<float>(sc_in.size()), *d_scout = B.get<float>(sc_out.size());
    int *d_igx = B.get<int>(nshot);
    float *d_wav = B.get<float>(nt);
    float2 *d_srcw = B.get<float2>(std::max(nwf, 1));
    int64_t *d_base = B.get<int64_t>(ntr), *d_zero = B.get<int64_t>(1);
    float *d_ux = B.get<float>(ntr * nt), *d_uz = B.get<float>(ntr * nt);
    float2 *d_sx = B.get<float2>(ntr * std::max(nwf, 1)), *d_sz = B.get<float2>(ntr * std::max(nwf, 1));
    float *d_mp = B.get<float>(nzx), *d_ms = B.get<float>(nzx);
    if (!d_po_p || !d_po_s || !d_vpm || !d_vsm || !d_pd_p || !d_pd_s || !d_tap || !d_tw || !d_wtab || !d_scin ||
        !d_scout || !d_igx || !d_wav || !d_srcw || !d_base || !d_zero || !d_ux || !d_uz || !d_sx || !d_sz || !d_mp ||
        !d_ms)
        return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
    std::vector<int64_t> base(ntr);
    for (size_t i = 0; i < ntr; i++) base[i] = (int64_t)((i / nmx) * nwf) * nmx + (int64_t)(i % nmx);
    const int64_t zero = 0;
    ECK(cudaMemcpyAsync(d_po_p, po_p.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_po_s, po_s.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_vpm, vpm.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_vsm, vsm.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_pd_p, pd_p.data(), sizeof(float) * nzx, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_pd_s, pd_s.data(), sizeof(float) * nzx, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_tap, taper.data(), sizeof(float) * nmx, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_wtab, wtab.data(), sizeof(float2) * nf, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_scin, sc_in.data(), sizeof(float) * sc_in.size(), cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_scout, sc_out.data(), sizeof(float) * sc_out.size(), cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_igx, igx.data(), sizeof(int) * nshot, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_wav, wav, sizeof(float) * nt, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_base, base.data(), sizeof(int64_t) * ntr, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_zero, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    if (adj) {
        ECK(cudaMemcpyAsync(d_ux, ux, sizeof(float) * ntr * nt, cudaMemcpyHostToDevice, st));
        ECK(cudaMemcpyAsync(d_uz, uz, sizeof(float) * ntr * nt, cudaMemcpyHostToDevice, st));
    } else {
        // the images to depth-major rows for the injection
        float *tmp = B.get<float>(nzx);
        if (!tmp) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
        ECK(cudaMemcpyAsync(tmp, mpp, sizeof(float) * nzx, cudaMemcpyHostToDevice, st));
        if (launch_transpose(tmp, nmx, nz, d_mp, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: transpose");
        ECK(cudaStreamSynchronize(st));
        ECK(cudaMemcpyAsync(tmp, mps2, sizeof(float) * nzx, cudaMemcpyHostToDevice, st));
        if (launch_transpose(tmp, nmx, nz, d_ms, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: transpose");
    }
    cudaEvent_t e0, e1;
    ECK(cudaEventCreate(&e0));
    ECK(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard()
        {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } eg{ e0, e1 };
    ECK(cudaEventRecord(e0, st));
    if (nwf > 0) {
        SpectraArgs sa{};
        // f_op's r2c of length (nw - 1) * 2 (ewem.c:465-471); with padt = 1 and an odd nt that is
        // one sample short of nt, and the reference writes past its buffer: the last sample is left out
        sa.d = d_wav; sa.ntr = 1; sa.nt = std::min(nt, nf); sa.ld = nt; sa.ntfft = nf; sa.ifmin = ifmin; sa.nwf = nwf;
        sa.out_base = d_zero; sa.out_fstride = 1; sa.wtab = d_wtab; sa.scale = d_scin; sa.out = d_srcw;
        if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: wavelet spectrum launch");
        if (adj) {
            sa.ntr = (int)ntr; sa.out_base = d_base; sa.out_fstride = nmx;
            sa.d = d_ux; sa.out = d_sx;
            if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: spectra launch");
            sa.d = d_uz; sa.out = d_sz;
            if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: spectra launch");
        }
    }
    EwemArgs a{};
    a.m.nmx = nmx; a.m.nz = nz; a.m.nref = 1; a.m.nwf = nwf; a.m.ifmin = ifmin; a.m.nshot = nshot;
    a.m.dw = dw; a.m.dz = p.dz; a.m.dkx = dkx; a.m.inv_n = 1.0f / (float)nkx; a.m.nlog = nkx;
    if (blu) {
        a.m.chirp = d_tw + chirp_off;
        a.m.bfft = d_tw + bfft_off;
    }
    a.nkx = nkx; a.gz = p.gz; a.sz = p.sz; a.oz = p.oz;
    a.inv_max_source = 1.f / max_source;
    a.inv_sqt = 1.f / sq;
    a.po_p = d_po_p; a.po_s = d_po_s; a.pd_p = d_pd_p; a.pd_s = d_pd_s; a.vp_mean = d_vpm; a.vs_mean = d_vsm;
    a.taper = d_tap; a.twid = d_tw; a.srcw = d_srcw; a.igx = d_igx; a.recv_x = d_sx; a.recv_z = d_sz;
    a.img_p = d_mp; a.img_s = d_ms; a.dg_x = d_sx; a.dg_z = d_sz;
    // the per-(frequency, depth) tables, in sub-bands of at most `chunk` frequencies when the
    // whole band's tables would take more than 4 GiB or a quarter of the free device memory
    const size_t rec_bytes = sizeof(float) * (size_t)EwemRec(nkx, nmx).floats() * nz;
    size_t free_b = 0, total_b = 0;
    ECK(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = std::min<size_t>((size_t)4 << 30, free_b / 4);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(nwf, 1), budget / rec_bytes));
    a.wbase = 0;
    a.nwc = std::min(nwf, chunk);
    const int nitems = nshot * a.nwc;  // the largest sub-band's items size the grid and the scratch
    const int per_cta = ewem_group(nfft, blu);  // shots per CTA: accumulator and source slots per CTA
    int grid = 0;
    size_t smem = 0;
    if (nitems > 0) {
        EwemArgs probe = a;  // sizing: no scratch yet
        if (ewem_launch(nfft, blu, adj, &probe, nsm, nitems, st, &grid, &smem))
            return set_error(WEM_ERR_SIZE, "wem_elastic: no kernel fits this row length and grid");
        a.tabs = B.get<float>(rec_bytes / sizeof(float) * a.nwc);
        if (!a.tabs) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
        if (adj) {
            a.slots = B.get<float2>(2 * (size_t)grid * per_cta * nzx);
            if (!a.slots) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
            ECK(cudaMemsetAsync(a.slots, 0, sizeof(float2) * 2 * (size_t)grid * per_cta * nzx, st));
        } else {
            a.smig = B.get<float2>((size_t)grid * per_cta * nzx);
            if (!a.smig) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
            ECK(cudaMemsetAsync(d_sx, 0, sizeof(float2) * ntr * nwf, st));
            ECK(cudaMemsetAsync(d_sz, 0, sizeof(float2) * ntr * nwf, st));
        }
        for (int w0 = 0; w0 < nwf; w0 += chunk) {
            a.wbase = w0;
            a.nwc = std::min(chunk, nwf - w0);
            wem_ewem_tables_kernel<<<a.nwc * nz, 256, 0, st>>>(a);
            ECK(cudaGetLastError());
            int g = 0;
            if (ewem_launch(nfft, blu, adj, &a, nsm, nshot * a.nwc, st, &g, &smem))
                return set_error(WEM_ERR_CUDA, "wem_elastic: depth kernel launch");
        }
    }
    if (adj) {
        if (nitems > 0) {
            if (launch_image_reduce(a.slots, grid * per_cta, nz, nmx, d_mp, st) ||
                launch_image_reduce(a.slots + (size_t)grid * per_cta * nzx, grid * per_cta, nz, nmx, d_ms, st))
                return set_error(WEM_ERR_CUDA, "wem_elastic: reduce launch");
        } else {
            ECK(cudaMemsetAsync(d_mp, 0, sizeof(float) * nzx, st));
            ECK(cudaMemsetAsync(d_ms, 0, sizeof(float) * nzx, st));
        }
    } else {
        SynthArgs sy{};
        sy.nwf = nwf; sy.ifmin = ifmin; sy.nt = nt; sy.nf = nf; sy.ntr = (int)ntr; sy.in_base = d_base;
        sy.in_fstride = nmx; sy.wtab = d_wtab; sy.scale = d_scout;
        sy.dg = d_sx; sy.out = d_ux;
        if (nwf > 0 && launch_synth(sy, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: synthesis launch");
        sy.dg = d_sz; sy.out = d_uz;
        if (nwf > 0 && launch_synth(sy, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: synthesis launch");
        if (nwf <= 0) {
            ECK(cudaMemsetAsync(d_ux, 0, sizeof(float) * ntr * nt, st));
            ECK(cudaMemsetAsync(d_uz, 0, sizeof(float) * ntr * nt, st));
        }
    }
    ECK(cudaEventRecord(e1, st));
    if (adj) {
        ECK(cudaMemcpyAsync(mpp, d_mp, sizeof(float) * nzx, cudaMemcpyDeviceToHost, st));
        ECK(cudaMemcpyAsync(mps2, d_ms, sizeof(float) * nzx, cudaMemcpyDeviceToHost, st));
    } else {
        ECK(cudaMemcpyAsync(ux, d_ux, sizeof(float) * ntr * nt, cudaMemcpyDeviceToHost, st));
        ECK(cudaMemcpyAsync(uz, d_uz, sizeof(float) * ntr * nt, cudaMemcpyDeviceToHost, st));
    }
    ECK(cudaStreamSynchronize(st));
    ECK(cudaEventElapsedTime(&g_last_ms, e0, e1));
    return WEM_OK;
}

extern "C" WEM_API float wem_elastic_last_ms(void) { return g_last_ms; }

// The reference's ewem() (ewem.h:3-16), one shot, float** rows as alloc2float builds them
// (seismic.c:92-106): adj = true, (ux, uz) -> (mpp, mps2) with mps1 = 0; adj = false, (mpp,
// mps2) -> (ux, uz) with uy = 0. The y component takes no part (ewem.c:553-741); nmy > 1
// runs the 3-D form.
extern "C" WEM_API int ewem(float **ux, float **uy, float **uz, float **mpp, float **mps1, float **mps2, float **wav,
                            int nt, float ot, float dt, int nmx, float omx, float dmx, int nmy, float omy, float dmy,
                            float sx, float sy, int nz, float oz, float dz, float gz, float sz, float **vp, float **vs,
                            float fmin, float fmax, int padt, int padx, bool adj, bool verbose)
{
    if (!ux || !uy || !uz || !mpp || !mps1 || !mps2 || !wav || !vp || !vs) return set_error(WEM_ERR_ARG, "ewem: null argument");
    wem_params p{};
    p.nt = nt; p.ot = ot; p.dt = dt; p.nmx = nmx; p.omx = omx; p.dmx = dmx; p.nmy = nmy; p.omy = omy; p.dmy = dmy;
    p.nz = nz; p.oz = oz; p.dz = dz; p.gz = gz; p.sz = sz; p.fmin = fmin; p.fmax = fmax; p.padt = padt; p.padx = padx;
    p.verbose = verbose ? 1 : 0;
    const size_t n = (size_t)nmx * nmy;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    // the rows of each float** array are contiguous (alloc2float: one block, row pointers into it)
    const int rc = wem_elastic(dev, &p, vp[0], vs[0], wav[0], 1, &sx, &sy, ux[0], uz[0], mpp[0], mps2[0], adj ? 1 : 0);
    if (rc) return rc;
    if (adj) memset(mps1[0], 0, sizeof(float) * n * nz);
    else memset(uy[0], 0, sizeof(float) * n * nt);
    return WEM_OK;
}
