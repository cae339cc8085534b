// C ABI of the GB300 TTV engine: argument validation with the reference's
// exact messages, the canonical-view planner, device scratch, dispatch and
// the host-buffer path.  Declarations: include/tlibg.h.
#include "../../include/tlibg.h"
#include "ttv_internal.h"
#include "ttv_kernels.cuh"
#include "ttv_device.cuh"
#include "ttv_general.cuh"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

using namespace tlibg;

namespace {

thread_local std::string t_last_error;
std::atomic<uint64_t> g_launches{0};
std::atomic<uint64_t> g_device_allocs{0};

// Every device allocation of the library goes through here (counted).
cudaError_t device_malloc(void** p, size_t bytes)
{
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) ++g_device_allocs;
    return e;
}

int fail(int code, const std::string& msg)
{
    t_last_error = msg;
    return code;
}

int ok()
{
    t_last_error.clear();
    return TLIBG_OK;
}

int cuda_fail(cudaError_t e, const char* where)
{
    std::string m = "tlibg: CUDA error in ";
    m += where;
    m += ": ";
    m += cudaGetErrorString(e);
    cudaGetLastError();   // clear a non-sticky error
    return fail(TLIBG_ERR_CUDA, m);
}

// --------------------------------------------------------------------------
// metadata predicates (shape.h, layout.h, strides.h of the reference)
// --------------------------------------------------------------------------
bool valid_shape(const size_t* n, size_t len)
{
    if (len == 0) return false;
    for (size_t r = 0; r < len; ++r)
        if (n[r] == 0) return false;
    return true;
}

bool valid_layout(const size_t* pi, size_t len)
{
    if (len == 0) return false;
    // a permutation of 1..len: every value in range and seen once
    std::vector<char> seen(len + 1, 0);
    for (size_t r = 0; r < len; ++r) {
        if (pi[r] == 0 || pi[r] > len || seen[pi[r]]) return false;
        seen[pi[r]] = 1;
    }
    return true;
}

// strides must not decrease along the layout (strides.h:76-101)
bool valid_strides(const size_t* pi, size_t len, const size_t* w)
{
    if (len == 1 && w[0] == 1) return true;
    for (size_t r = 0; r + 1 < len; ++r)
        if (w[pi[r] - 1] > w[pi[r + 1] - 1]) return false;
    return true;
}

bool shape_is_scalar(const size_t* n, size_t len)
{
    for (size_t r = 0; r < len; ++r)
        if (n[r] != 1) return false;
    return true;
}

bool shape_is_vector(const size_t* n, size_t len)
{
    if (len == 1) return n[0] > 1;
    bool gt = n[0] > 1 || n[1] > 1, eq = n[0] == 1 || n[1] == 1;
    for (size_t r = 2; r < len; ++r)
        if (n[r] != 1) return false;
    return gt && eq;
}

// dense strides of (n, pi), with the reference's convention that vectors and
// scalars get all-ones strides (strides.h:31-57)
void dense_strides(const size_t* n, const size_t* pi, size_t p, size_t* w)
{
    for (size_t r = 0; r < p; ++r) w[r] = 1;
    if (shape_is_vector(n, p) || shape_is_scalar(n, p)) return;
    for (size_t r = 1; r < p; ++r) w[pi[r] - 1] = w[pi[r - 1] - 1] * n[pi[r - 1] - 1];
}

const char* const MSG[] = {
    "",
    "Error in tlib::tensor_times_vector: input tensor order should be greater zero.",
    "Error in tlib::tensor_times_vector: contraction mode should be greater zero or less than or equal to p.",
    "Error in tlib::tensor_times_vector: pointer to input tensor A should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input vector B should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor C should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor shape vector na should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input vector shape vector nb should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor shape vector nc should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor stride vector wa should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor stride vector wc should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to input tensor permutation vector pia should not be zero.",
    "Error in tlib::tensor_times_vector: pointer to output tensor permutation vector pic should not be zero.",
    "Error in tlib::tensor_times_vector: contraction dimension of A and B are not equal.",
    "Error in tlib::tensor_times_vector: shape vector of A is not valid.",
    "Error in tlib::tensor_times_vector: shape vector of C is not valid.",
    "Error in tlib::tensor_times_vector: layout vector of A is not valid.",
    "Error in tlib::tensor_times_vector: layout vector of C is not valid.",
    "Error in tlib::tensor_times_vector: stride vector of A is not valid.",
    "Error in tlib::tensor_times_vector: stride vector of C is not valid.",
    "Error in tlib::detail::compute_inverse_pia_m: beginning of layout tuples of both tensors are not correct.",
    "Error in tlib::detail::compute_inverse_pia_m: end of layout tuples of both tensors are not correct.",
};

// The reference's checks in its order (ttv.h:64-89).
int check_call(size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
               const size_t* pia, const void* b, const size_t* nb, const void* c, const size_t* nc,
               const size_t* wc, const size_t* pic)
{
    if (p == 0) return 1;
    if (q == 0 || q > p) return 2;
    if (!a) return 3;
    if (!b) return 4;
    if (!c) return 5;
    if (!na) return 6;
    if (!nb) return 7;
    if (!nc) return 8;
    if (!wa) return 9;
    if (!wc) return 10;
    if (!pia) return 11;
    if (!pic) return 12;
    if (na[q - 1] != nb[0]) return 13;
    if (!valid_shape(na, p)) return 14;
    if (!valid_shape(nc, p - 1)) return 15;
    if (!valid_layout(pia, p)) return 16;
    if (!valid_layout(pic, p - 1)) return 17;
    if (!valid_strides(pia, p, wa)) return 18;
    if (!valid_strides(pic, p - 1, wc)) return 19;
    return 0;
}

// pic must be the layout that pia induces once mode q is removed
// (tensor_times_vector.h:147-168); only the reference's case 8 checks it.
int check_pic(const size_t* pia, const size_t* pic, size_t p, size_t q)
{
    size_t k = 0;
    while (k < p && pia[k] != q) ++k;
    for (size_t i = 0; i < k; ++i)
        if ((pia[i] > q && pic[i] + 1 != pia[i]) || (pia[i] < q && pic[i] != pia[i])) return 20;
    for (size_t i = k; i + 1 < p; ++i)
        if ((pia[i + 1] > q && pic[i] + 1 != pia[i + 1]) || (pia[i + 1] < q && pic[i] != pia[i + 1])) return 21;
    return 0;
}

bool mul_overflows(uint64_t x, uint64_t y, uint64_t* r)
{
    if (x != 0 && y > (uint64_t(1) << 62) / x) return true;
    *r = x * y;
    return false;
}

struct Canon {
    uint64_t P = 1, nq = 1, S = 1;
    int ref_case = 0;
};

// Validate a call and reduce it to the canonical (S, nq, P) view.
int analyse(size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
            const size_t* pia, const void* b, const size_t* nb, const void* c, const size_t* nc,
            const size_t* wc, const size_t* pic, Canon* out)
{
    const int code = check_call(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
    if (code) return fail(TLIBG_ERR_ARGUMENT, MSG[code]);

    // reference case (cases.h:24-36); p == 1 never reaches here (C's shape is empty)
    int kase;
    if (p == 2)
        kase = (q == 1) ? (pia[0] == 1 ? 2 : 4) : (pia[0] == 1 ? 3 : 5);
    else if (pia[0] == q)
        kase = 6;
    else if (pia[p - 1] == q)
        kase = 7;
    else
        kase = 8;
    if (kase == 8) {
        const int pc = check_pic(pia, pic, p, q);
        if (pc) return fail(TLIBG_ERR_ARGUMENT, MSG[pc]);
    }

    Canon cn;
    cn.ref_case = kase;
    size_t k = 0;
    while (pia[k] != q) ++k;
    uint64_t total = 1;
    for (size_t r = 0; r < p; ++r)
        if (mul_overflows(total, na[r], &total))
            return fail(TLIBG_ERR_UNSUPPORTED, "tlibg: the number of elements of A exceeds 2^62");
    for (size_t r = 0; r < k; ++r) cn.P *= na[pia[r] - 1];
    for (size_t r = k + 1; r < p; ++r) cn.S *= na[pia[r] - 1];
    cn.nq = na[q - 1];

    // A must be dense in its layout: every mode with extent > 1 carries the
    // stride the reference's generate_strides gives it.
    std::vector<size_t> w(p), running(p);
    {
        size_t acc = 1;
        for (size_t r = 0; r < p; ++r) {
            running[pia[r] - 1] = acc;
            acc *= na[pia[r] - 1];
        }
        for (size_t r = 0; r < p; ++r)
            if (na[r] > 1 && wa[r] != running[r])
                return fail(TLIBG_ERR_UNSUPPORTED,
                            "tlibg: the gpu policy requires a dense tensor A: stride vector wa does "
                            "not match the shape and layout (as generate_strides makes them)");
    }
    // In case 8 the reference addresses C through wc: it must be dense too.
    // (Cases 2-7 write C in canonical order and ignore nc, wc and pic.)
    if (kase == 8) {
        std::vector<size_t> ncx;
        for (size_t r = 0; r < p; ++r)
            if (r != q - 1) ncx.push_back(na[r]);
        size_t acc = 1;
        std::vector<size_t> run(p - 1);
        for (size_t r = 0; r + 1 < p; ++r) {
            run[pic[r] - 1] = acc;
            acc *= ncx[pic[r] - 1];
        }
        for (size_t r = 0; r + 1 < p; ++r)
            if (ncx[r] > 1 && wc[r] != run[r])
                return fail(TLIBG_ERR_UNSUPPORTED,
                            "tlibg: the gpu policy requires a dense tensor C: stride vector wc does "
                            "not match the output shape and layout");
    }
    *out = cn;
    return TLIBG_OK;
}

// --------------------------------------------------------------------------
// device properties
// --------------------------------------------------------------------------
struct DevInfo {
    int sms = 0;
    bool ok = false;
};

DevInfo dev_info()
{
    static std::mutex mu;
    static std::map<int, DevInfo> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return DevInfo{};
    }
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    DevInfo d;
    if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) d.ok = true;
    else cudaGetLastError();
    cache[dev] = d;
    return d;
}

// --------------------------------------------------------------------------
// planner
// --------------------------------------------------------------------------
size_t elem_size_a(int dt) { return dt == F64 ? 8 : (dt == BF16A ? 2 : 4); }
size_t elem_size_t(int dt) { return dt == F64 ? 8 : 4; }
bool aligned(const void* p, size_t n) { return (reinterpret_cast<uintptr_t>(p) % n) == 0; }
uint64_t cdiv(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
int pow2_floor(uint64_t x)
{
    int r = 1;
    while ((uint64_t)r * 2 <= x && r < (1 << 30)) r *= 2;
    return r;
}

// Streamed kernel: A as rows of L contiguous elements, R rows per 16 KB chunk,
// a static block of units per CTA (row form: rows; column form: (s, segment)).
#ifndef TLIBG_SCALAR_OUTPUTS
#define TLIBG_SCALAR_OUTPUTS 2
#endif

int make_stream_plan(Plan pl, const Canon& cn, const tlibg_options* opt, int sms, Plan* out)
{
    const size_t ea = elem_size_a(pl.dtype);
    pl.kind = KIND_STREAM;
    pl.stream_col = cn.P > 1 ? 1 : 0;
    pl.vec = 1;
    pl.L = cn.P == 1 ? cn.nq : cn.P;
    pl.R = std::max<uint64_t>(1, (uint64_t)STREAM_STAGE_BYTES / (pl.L * ea));
    const int force_split = opt ? opt->split : 0;
    const int force_group = opt ? opt->group : 0;
    if (!pl.stream_col) {
        // fp64 rows: at least 32 elements per lane, so the DADDs of the shuffle tree stay
        // small next to the one DFMA per element (GB300's FP64 pipe is the bound there)
        const uint64_t per_lane = pl.dtype == F64 ? 32 : 8;
        int G = force_group > 0 ? force_group : std::min(32, std::max(1, pow2_floor(pl.L / per_lane)));
        if (G < 1 || G > 32 || (G & (G - 1)))
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: lanes per row must be a power of two in 1..32");
        pl.group = G;
    } else {
        pl.group = 1;
        pl.RG = cn.P < (uint64_t)STREAM_CONSUMERS ? (int)(STREAM_CONSUMERS / cn.P) : 1;
        pl.J = cn.P < (uint64_t)STREAM_CONSUMERS ? 1 : (int)cdiv(cn.P, STREAM_CONSUMERS);
    }
    const int cps = std::max(1, plan_ctas_per_sm(pl));
    const uint64_t grid_max = (uint64_t)sms * cps;
    uint64_t nseg = 1;
    if (!pl.stream_col) {
        pl.units = cn.S;
    } else {
        if (force_split > 0) {
            nseg = (uint64_t)force_split;
        } else if (cn.S < 2 * grid_max) {
            nseg = cdiv(2 * grid_max, cn.S);
            nseg = std::min<uint64_t>(nseg, std::max<uint64_t>(1, cn.nq / (2 * pl.R)));
        }
        nseg = std::max<uint64_t>(1, std::min<uint64_t>(nseg, cn.nq));
        pl.seg_len = cdiv(cn.nq, nseg);
        nseg = cdiv(cn.nq, pl.seg_len);
        pl.units = cn.S * nseg;
    }
    pl.split = (int)nseg;
    pl.units_per_cta = cdiv(pl.units, std::min<uint64_t>(grid_max, pl.units));
    pl.grid = (int)cdiv(pl.units, pl.units_per_cta);
    pl.f64_combine = (pl.dtype != F64) && pl.split > 1 && cn.nq > (uint64_t(1) << 20);
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

// Plan hints installed by the autotuner: (type, P, n_q, S) -> options used when
// the caller leaves every kernel choice to the planner.
std::mutex g_hint_mu;
std::map<std::tuple<int, uint64_t, uint64_t, uint64_t>, tlibg_options> g_hints;

bool default_choices(const tlibg_options* opt)
{
    return !opt || (opt->kind < 0 && opt->group == 0 && opt->vec == 0 && opt->split == 0 &&
                    opt->accumulate == TLIBG_ACC_COMPENSATED);
}

int make_plan_inner(int dtype, const Canon& cn, const void* a, const void* b, const tlibg_options* opt,
                    int sms, Plan* out);

int make_plan(int dtype, const Canon& cn, const void* a, const void* b, const tlibg_options* opt,
              int sms, Plan* out)
{
    if (default_choices(opt)) {
        tlibg_options hinted;
        bool found = false;
        {
            std::lock_guard<std::mutex> lk(g_hint_mu);
            auto it = g_hints.find(std::make_tuple(dtype, cn.P, cn.nq, cn.S));
            if (it != g_hints.end()) {
                hinted = it->second;
                found = true;
            }
        }
        if (found) {
            hinted.sync = opt ? opt->sync : 0;
            Plan tmp;
            // a hint that no longer applies (e.g. narrower alignment) falls back to the rules
            if (make_plan_inner(dtype, cn, a, b, &hinted, sms, &tmp) == TLIBG_OK) {
                *out = tmp;
                return TLIBG_OK;
            }
        }
    }
    return make_plan_inner(dtype, cn, a, b, opt, sms, out);
}

// TMA-staged column kernel: items (segment, slice, tile of 4 KB of a row), a
// contiguous block of items per CTA; q is split only to fill the grid.
int make_col_bulk_plan(Plan pl, const Canon& cn, const tlibg_options* opt, int sms, Plan* out)
{
    pl.kind = KIND_COL_BULK;
    pl.group = 1;
    pl.vec = (int)(col_bulk_tile(pl.dtype) / CB_CONSUMERS);
    const uint64_t ntiles = cdiv(cn.P, col_bulk_tile(pl.dtype));
    const uint64_t tiles = cn.S * ntiles;
    const uint64_t bmax = BSTAGE_BYTES / elem_size_t(pl.dtype);
    const int cps = std::max(1, plan_ctas_per_sm(pl));
    const uint64_t grid_full = (uint64_t)sms * cps;
    const int force_split = opt ? opt->split : 0;
    uint64_t nseg = cdiv(cn.nq, bmax);
    if (force_split > 0) {
        if ((uint64_t)force_split < nseg)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: forced split leaves a segment longer than the staged b buffer");
        nseg = (uint64_t)force_split;
    } else if (tiles < 2 * grid_full) {
        nseg = std::max<uint64_t>(nseg, std::min<uint64_t>(cdiv(2 * grid_full, tiles),
                                                           std::max<uint64_t>(1, cn.nq / (4 * CB_RB))));
    }
    nseg = std::max<uint64_t>(1, std::min<uint64_t>(nseg, cn.nq));
    const uint64_t seg_len = cdiv(cn.nq, nseg);
    nseg = cdiv(cn.nq, seg_len);
    pl.split = (int)nseg;
    pl.seg_len = seg_len;
    pl.items = tiles * nseg;
    const uint64_t grid = std::min<uint64_t>(grid_full, pl.items);
    pl.items_per_cta = cdiv(pl.items, grid);
    pl.grid = (int)cdiv(pl.items, pl.items_per_cta);
    pl.f64_combine = (pl.dtype != F64) && pl.split > 1 && cn.nq > (uint64_t(1) << 20);
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

// Row-tile kernel: tiles of 32 R rows (R rows per lane), a static round robin
// of tiles over the warps of a grid of resident CTAs.
int make_row_tile_plan(Plan pl, const Canon& cn, const tlibg_options* opt, int sms, Plan* out)
{
    if (opt && opt->split > 1)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-tile kernel does not split the contracted mode");
    pl.kind = KIND_ROW_TILE;
    pl.group = 1;
    pl.vec = 1;
    pl.split = 1;
    pl.seg_len = cn.nq;
    pl.items = cn.S;
    pl.rows_m = rowt_rows_per_lane(cn.nq, elem_size_a(pl.dtype));
    const int cps = std::max(1, plan_ctas_per_sm(pl));
    const uint64_t tiles = cdiv(cn.S, 32 * (uint64_t)pl.rows_m);
    pl.grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * cps, cdiv(tiles, ROWT_WARPS)));
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

// Row-panel kernel: items (segment of b, block of rows); row blocks only as
// many as it takes to give the grid about two items per CTA.
// Rows in flight: two for fp32 (64 registers, no spill); one for fp64 and
// bf16-stored A, whose second row spills.
#ifndef TLIBG_ROW_PANEL_RR
#define TLIBG_ROW_PANEL_RR(dtype) ((dtype) == F32 ? 2 : 1)
#endif
int make_row_panel_plan(Plan pl, const Canon& cn, const tlibg_options* opt, int sms, Plan* out)
{
    const int vmax = (int)(16 / elem_size_a(pl.dtype));
    if (opt && opt->vec > 0 && opt->vec != vmax)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-panel kernel loads 16 bytes per vector");
    if (opt && opt->split > 0)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-panel kernel splits the contracted mode into "
                                        "segments of its own");
    const int rr = (opt && opt->group > 0) ? opt->group : TLIBG_ROW_PANEL_RR(pl.dtype);
    if (rr != 1 && rr != 2)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: rows in flight of the row-panel kernel must be 1 or 2");
    pl.kind = KIND_ROW_PANEL;
    pl.vec = vmax;
    pl.group = rr;
    pl.rows_m = rr;
    const uint64_t L = row_panel_seg(pl.dtype);
    const uint64_t nseg = cdiv(cn.nq, L);
    const int cps = std::max(1, plan_ctas_per_sm(pl));
    const uint64_t grid_full = (uint64_t)sms * cps;
    uint64_t nrb = 1;
    if (nseg < 2 * grid_full) nrb = std::min<uint64_t>(cn.S, cdiv(2 * grid_full, nseg));
    const uint64_t rbk = cdiv(cn.S, nrb);
    nrb = cdiv(cn.S, rbk);
    pl.seg_len = L;
    pl.split = (int)nseg;
    pl.items = nseg * nrb;
    pl.items_per_cta = rbk;
    pl.grid = (int)std::min<uint64_t>(grid_full, pl.items);
    pl.f64_combine = (pl.dtype != F64) && cn.nq > (uint64_t(1) << 20);
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

// Rows that are not whole 16-byte vectors: the row-shift kernel (aligned
// vector bodies against shifted copies of b in shared memory), G lanes per row
// by the row kernel's rule, no split.
int make_row_shift_plan(Plan pl, const Canon& cn, const tlibg_options* opt, int sms, Plan* out)
{
    const int vmax = (int)(16 / elem_size_a(pl.dtype));
    if (opt && opt->vec > 0 && opt->vec != vmax)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-shift kernel loads 16 bytes per vector");
    if (opt && opt->split > 1)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-shift kernel does not split the contracted mode");
    int G;
    if (pl.dtype == F64)
        G = std::max(2, std::min(32, pow2_floor(std::max<uint64_t>(1, cn.nq / 64))));
    else
        G = std::max(2, std::min(32, pow2_floor(std::max<uint64_t>(1, cn.nq / 4 / 16))));
    if (opt && opt->group > 0) G = opt->group;
    if (G < 1 || G > 32 || (G & (G - 1)))
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: lanes per row must be a power of two in 1..32");
    pl.kind = KIND_ROW_SHIFT;
    pl.vec = vmax;
    pl.group = G;
    pl.split = 1;
    pl.seg_len = cn.nq;
    pl.items = cn.S;
    pl.items_per_cta = 0;
    const int cps = std::max(1, plan_ctas_per_sm(pl));
    pl.grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * cps, cdiv(cn.S, BLOCK / G)));
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

int make_plan_inner(int dtype, const Canon& cn, const void* a, const void* b, const tlibg_options* opt,
                    int sms, Plan* out)
{
    Plan pl;
    pl.dtype = dtype;
    pl.sms = sms;
    pl.P = cn.P;
    pl.nq = cn.nq;
    pl.S = cn.S;
    // fp32: Kahan unless plain is asked for.  fp64: the register kernels mix native
    // DFMA with double-float emulation on the FP32/INT32 pipes (measured faster than
    // DFMA alone on GB300); the streamed kernel uses native DFMA unless the emulation
    // is asked for (TLIBG_ACC_DOUBLE_FLOAT); TLIBG_ACC_PLAIN is native DFMA everywhere.
    if (dtype == F64)
        pl.kahan = (opt && opt->accumulate == TLIBG_ACC_PLAIN) ? 0 : 1;
    else
        pl.kahan = (opt && opt->accumulate == TLIBG_ACC_PLAIN) ? 0 : 1;
    pl.kind = cn.P == 1 ? KIND_ROW : KIND_COL;
    const size_t ea = elem_size_a(dtype), et = elem_size_t(dtype);
    const bool eligible = stream_eligible(dtype, cn.P, cn.nq);
    if (opt && opt->kind == KIND_STREAM && !eligible)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the streamed kernel needs whole rows of the canonical view "
                                        "(n_q when P == 1, else P) within one 16 KB stage");
    const bool realign_ok = cn.P > 1 && dtype != BF16A;
    if (opt && opt->kind == KIND_COL_REALIGN && !realign_ok)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the realigning column kernel needs prefix P > 1 and "
                                        "fp32 or fp64 A");
    if (opt && opt->kind == KIND_COL_THIN && cn.P == 1)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the thin-prefix column kernel needs prefix P > 1");
    const bool row_tile_ok = cn.P == 1 && cn.nq <= (uint64_t)ROWT_MAX_NQ;
    if (opt && opt->kind == KIND_ROW_TILE && !row_tile_ok)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-tile kernel needs prefix P == 1 and n_q <= 64");
    if (opt && opt->kind == KIND_COL_BULK && cn.P == 1)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: the TMA-staged column kernel needs prefix P > 1");
    if (opt && opt->kind == KIND_COL_BULK) return make_col_bulk_plan(pl, cn, opt, sms, out);
    // Long q-fastest rows with 16-byte loads (at least two segments of b): the
    // row-panel kernel holds b's segment in registers across a block of rows.
    // On request only: measured on GB300 against the row kernel (whose
    // segment-major walk already has the rows of one b segment read together)
    // on the asymmetric sweep's q = 1 rows, 10 back-to-back launches each:
    // 4 x 2^26 floats 4.45 (rows in flight 1) / 4.37 (2) against 4.89 TB/s,
    // 16 x 2^24 6.02 / 6.11 against 6.05, 64 x 2^22 5.80 / 5.88 against 6.10,
    // 256 x 2^20 5.14 / 5.29 against 6.12.
    const bool panel_ok = cn.P == 1 && cn.nq % (16 / ea) == 0 && aligned(a, 16) && aligned(b, 16) &&
                          cn.nq > row_panel_seg(dtype);
    if (opt && opt->kind == KIND_ROW_PANEL) {
        if (!panel_ok)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-panel kernel needs prefix P == 1, rows of "
                                            "16-byte vectors on 16-byte aligned A and b, and n_q longer "
                                            "than one segment of b");
        return make_row_panel_plan(pl, cn, opt, sms, out);
    }
    const bool shift_ok = cn.P == 1 && dtype != BF16A &&
                          rs_smem_bytes(cn.nq, et, dtype == F64 && pl.kahan) <= RS_SMEM_MAX;
    if (opt && opt->kind == KIND_ROW_SHIFT) {
        if (!shift_ok)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: the row-shift kernel needs prefix P == 1, fp32 or fp64 A, "
                                            "and b's shifted copies within 48 KB of shared memory");
        return make_row_shift_plan(pl, cn, opt, sms, out);
    }
    if (opt && opt->kind >= 0 && opt->kind != KIND_STREAM && opt->kind != KIND_COL_REALIGN &&
        opt->kind != KIND_COL_THIN && opt->kind != KIND_ROW_TILE && opt->kind != pl.kind)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: forced kernel kind does not match the problem "
                                        "(row kernel needs prefix P == 1, column kernel P > 1)");
    // Default for q-fastest rows: the register row kernel, except the short rows below.
    // The streamed kernel (row and column forms) stays available on request.
    bool rows_aligned = false;
    {
        const size_t vb = 16 / ea;
        rows_aligned = cn.nq % vb == 0 && aligned(a, 16) && aligned(b, 16);
    }
    // Short q-fastest rows take the row-tile kernel (measured on GB300 against the
    // register row kernel and the streamed kernel): fp64 rows of at most 32 elements
    // with the double-float mix (rows of 16 / 25: 5.2-5.4 vs 4.0-4.1 TB/s; from 40
    // elements on the row kernel's lane pairs win), and fp32 / bf16 rows under 64
    // elements that are not 16-byte aligned (rows of 25: 5.5 vs 4.2 TB/s streamed).
    // fp64 rows under 8 elements accumulate with native DFMA only there: the mix's
    // per-row fold costs more than it saves (rows of 3: 4.6 vs 3.2 TB/s).
    const bool no_split = !(opt && opt->split > 1);
    const bool row_tile_default =
        row_tile_ok && no_split &&
        ((dtype == F64 && pl.kahan && cn.nq <= 32) || (dtype != F64 && !rows_aligned && cn.nq < 64));
    if ((opt && opt->kind == KIND_ROW_TILE) || (row_tile_default && !(opt && opt->kind >= 0))) {
        if (dtype == F64 && cn.nq < 8 && !(opt && opt->accumulate == TLIBG_ACC_DOUBLE_FLOAT)) pl.kahan = 0;
        return make_row_tile_plan(pl, cn, opt, sms, out);
    }
    if (opt && opt->kind == KIND_STREAM) {
        if (dtype == F64) pl.kahan = (opt && opt->accumulate == TLIBG_ACC_DOUBLE_FLOAT) ? 1 : 0;
        return make_stream_plan(pl, cn, opt, sms, out);
    }
    // Rows of 64 or more elements that are not whole 16-byte vectors (or A off the
    // 16-byte grid), with enough rows to fill the lane groups without a split: the
    // row-shift kernel instead of the row kernel's scalar loads (measured on GB300
    // for the sweep's rows of 645 floats / doubles).
    if (shift_ok && !rows_aligned && cn.nq >= 64 && no_split && !(opt && (opt->kind >= 0 || opt->vec > 0))) {
        Plan sp;
        if (make_row_shift_plan(pl, cn, opt, sms, &sp) == TLIBG_OK) {
            // at least four rounds of rows over the resident lane groups (the kernel
            // has no split to fill the GPU with fewer rows)
            const uint64_t groups = (uint64_t)sms * std::max(1, plan_ctas_per_sm(sp)) * (BLOCK / sp.group);
            if (cn.S >= 4 * groups) {
                *out = sp;
                return TLIBG_OK;
            }
        }
    }
    const int vmax = (int)(16 / ea);

    // vector width: the widest load that keeps every access aligned
    int V = (opt && opt->vec > 0) ? opt->vec : vmax;
    if (V > vmax || (V & (V - 1)))
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: vector width must be a power of two up to 16 bytes");
    auto vec_ok = [&](int v) {
        if (pl.kind == KIND_ROW)
            return cn.nq % v == 0 && aligned(a, v * ea) && aligned(b, std::min<size_t>(16, v * et));
        return cn.P % v == 0 && aligned(a, v * ea);
    };
    if (opt && opt->kind == KIND_COL_REALIGN) {
        if (opt->vec > 0 && opt->vec != vmax)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: the realigning column kernel loads 16 bytes per vector");
        V = vmax;
        pl.kind = KIND_COL_REALIGN;
    } else if (opt && opt->vec > 0) {
        if (!vec_ok(V)) return fail(TLIBG_ERR_ARGUMENT, "tlibg: forced vector width violates alignment");
    } else {
        while (V > 1 && !vec_ok(V)) V /= 2;
        // The realigning kernel (16-byte loads realigned by shuffles) stays available on
        // request: since scalar loads carry two outputs per thread (the strided kernel)
        // they measure ahead of it for every unaligned prefix of the sweeps.
        const bool realign_default = false;
        if (V < vmax && realign_ok && !(opt && opt->kind >= 0) && realign_default) {
            V = vmax;
            pl.kind = KIND_COL_REALIGN;
        }
    }
    pl.vec = V;

    const int force_split = opt ? opt->split : 0;
    const int force_group = opt ? opt->group : 0;
    if (pl.kind == KIND_ROW) {
        // Lanes per row, measured on GB300: fp32 about 16 vector loads per lane (64
        // elements with scalar loads; at least 2 lanes); fp64 about 64 elements per lane
        // (at least 2 lanes), one lane for rows of at most 32 elements.
        const uint64_t nvec = cdiv(cn.nq, V);
        int Gdef;
        if (dtype == F64)
            Gdef = cn.nq <= 32 ? 1 : std::max(2, std::min(32, pow2_floor(std::max<uint64_t>(1, cn.nq / 64))));
        else if (V == 1)   // scalar loads: about 64 elements per lane
            Gdef = std::max(2, std::min(32, pow2_floor(std::max<uint64_t>(1, cn.nq / 64))));
        else
            Gdef = std::max(2, std::min(32, pow2_floor(std::max<uint64_t>(1, nvec / 16))));
        int G = force_group > 0 ? force_group : Gdef;
        if (G < 1 || G > 32 || (G & (G - 1)))
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: lanes per row must be a power of two in 1..32");
        pl.group = G;
        const int cps = std::max(1, plan_ctas_per_sm(pl));
        const uint64_t slots = (uint64_t)sms * cps * (BLOCK / G);
        uint64_t nseg = 1;
        if (force_split > 0) {
            nseg = (uint64_t)force_split;
        } else if (cn.S < 2 * slots) {
            // Lane groups take the (row, segment) items round-robin, so a launch lasts
            // ceil(items / slots) rounds of one segment each.  Two rounds is the rule;
            // another round count r in 1..4 (with the most segments that fill r rounds)
            // replaces it when rounds x segment length drops by more than 2 %: 1024 rows
            // of 2^18 floats at 32 lanes took 10 segments = 3 rounds, the third a tenth
            // full (5.04 TB/s), where 9 fill two.
            const uint64_t min_len = (uint64_t)V * G * 4;
            const uint64_t max_seg = std::max<uint64_t>(1, cn.nq / min_len);
            auto cost = [&](uint64_t ns) { return cdiv(cn.S * ns, slots) * cdiv(cn.nq, ns); };
            uint64_t best = std::max<uint64_t>(1, std::min<uint64_t>(max_seg, (2 * slots) / cn.S));
            const uint64_t base = cost(best);
            for (uint64_t r = 1; r <= 4; ++r) {
                const uint64_t ns = std::min<uint64_t>(max_seg, (r * slots) / cn.S);
                if (ns >= 1 && (double)cost(ns) < 0.98 * (double)base && cost(ns) < cost(best)) best = ns;
            }
            nseg = best;
        } else if (cn.S < 16 * slots) {
            // Many rows, but few rounds of them: 16384 rows over 4864 lane groups take 4
            // rounds, the last a third full.  Two to four segments per row fill the rounds
            // better (2 segments: 7 rounds of half rows, 12.5 % less); taken when they cut
            // rounds x segment length by more than 2 %.
            const uint64_t min_len = (uint64_t)V * G * 16;
            auto cost = [&](uint64_t ns) { return cdiv(cn.S * ns, slots) * cdiv(cn.nq, ns); };
            const uint64_t base = cost(1);
            for (uint64_t ns = 2; ns <= 4; ++ns)
                if (cn.nq / ns >= min_len && (double)cost(ns) < 0.98 * (double)base && cost(ns) < cost(nseg))
                    nseg = ns;
        }
        nseg = std::max<uint64_t>(1, std::min<uint64_t>(nseg, cn.nq));
        uint64_t seg_len = cdiv(cn.nq, nseg);
        seg_len = cdiv(seg_len, V) * V;
        nseg = cdiv(cn.nq, seg_len);
        pl.split = (int)nseg;
        pl.seg_len = seg_len;
        pl.items = cn.S * nseg;
        // rows of at most two vectors per lane: the short-row kernel keeps several rows
        // per lane group in flight (measured on GB300 for fp32 / bf16 storage; fp64 rows
        // that short are bound by their per-row reductions on the FP64 pipe instead)
        if (nseg == 1 && cn.nq % V == 0 && dtype != F64) {
            const uint64_t nv = cn.nq / V;
            pl.rows_m = nv <= (uint64_t)G ? 1 : (nv <= 2 * (uint64_t)G ? 2 : 0);
        }
        const uint64_t groups_per_cta = BLOCK / G;
        pl.grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * cps, cdiv(pl.items, groups_per_cta)));
        pl.items_per_cta = 0;
    } else {
        const uint64_t outputs = cn.S * cn.P;
        const uint64_t bmax = BSTAGE_BYTES / et;
        // thin prefix: P / V lanes cover a row and divide the warp
        const uint64_t PV = cn.P / V;
        const bool thin_shape = pl.kind == KIND_COL && cn.P % V == 0 && PV <= 32 && 32 % PV == 0;
        if (opt && opt->kind == KIND_COL_THIN && !thin_shape)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: the thin-prefix column kernel needs P / vector width "
                                            "to divide 32");
        bool thin = opt && opt->kind == KIND_COL_THIN;
        if (!thin && thin_shape && !(opt && opt->kind >= 0)) {
            // few outputs: the plain column kernel would leave most lanes idle
            const uint64_t TO1 = (uint64_t)(BLOCK / 32) * 32 * V;
            Plan probe = pl;
            probe.group = 1;
            thin = cdiv(outputs, TO1) < (uint64_t)sms * std::max(1, plan_ctas_per_sm(probe));
        }
        if (thin) {
            pl.kind = KIND_COL_THIN;
            pl.group = 1;
            const int cps = std::max(1, plan_ctas_per_sm(pl));
            const uint64_t grid_full = (uint64_t)sms * cps;
            const uint64_t RG = 32 / PV;
            const uint64_t min_len = (BLOCK / 32) * RG * 4;   // four loads per lane at least
            uint64_t nseg = cdiv(cn.nq, bmax);
            if (force_split > 0) {
                if ((uint64_t)force_split < nseg)
                    return fail(TLIBG_ERR_ARGUMENT, "tlibg: forced split leaves a segment longer than the staged b buffer");
                nseg = (uint64_t)force_split;
            } else if (cn.S * nseg < 2 * grid_full) {
                nseg = std::max<uint64_t>(nseg, std::min<uint64_t>(cdiv(2 * grid_full, cn.S),
                                                                   std::max<uint64_t>(1, cn.nq / min_len)));
            }
            nseg = std::max<uint64_t>(1, std::min<uint64_t>(nseg, cn.nq));
            const uint64_t seg_len = cdiv(cn.nq, nseg);
            nseg = cdiv(cn.nq, seg_len);
            pl.split = (int)nseg;
            pl.seg_len = seg_len;
            pl.items = cn.S * nseg;
            const uint64_t grid = std::min<uint64_t>(grid_full, pl.items);
            pl.items_per_cta = cdiv(pl.items, grid);
            pl.grid = (int)cdiv(pl.items, pl.items_per_cta);
            pl.f64_combine = (dtype != F64) && pl.split > 1 && cn.nq > (uint64_t(1) << 20);
            pl.smem = plan_smem_bytes(pl);
            *out = pl;
            return TLIBG_OK;
        }
        // contractions of at most CS_MAXQ rows with vector loads: the short-contraction
        // kernel (two tiles per thread, every row of both loaded before any product)
        if (pl.kind == KIND_COL && V > 1 && dtype != BF16A && cn.nq <= (uint64_t)CS_MAXQ && force_group <= 1 &&
            force_split <= 1) {
            pl.rows_m = 1;
            pl.group = 1;
            pl.split = 1;
            pl.seg_len = cn.nq;
            const int cps = std::max(1, plan_ctas_per_sm(pl));
            const uint64_t tiles = cdiv(cn.S * cn.P, (uint64_t)BLOCK * V);
            pl.items = cdiv(tiles, 2);
            const uint64_t grid = std::min<uint64_t>((uint64_t)sms * cps, pl.items);
            pl.items_per_cta = cdiv(pl.items, grid);
            pl.grid = (int)cdiv(pl.items, pl.items_per_cta);
            pl.smem = plan_smem_bytes(pl);
            *out = pl;
            return TLIBG_OK;
        }
        int WI = force_group > 0 ? force_group : 1;
        if (WI != 1 && WI != 2 && WI != 4 && WI != 8)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: warps along the contracted mode must be 1, 2, 4 or 8");
        // scalar loads: several outputs per thread, 32 apart (more loads in flight per row)
        if (pl.kind == KIND_COL && V == 1) pl.mo = TLIBG_SCALAR_OUTPUTS;
        auto tiles_for = [&](int wi) { return cdiv(outputs, (uint64_t)((BLOCK / 32) / wi) * 32 * V * pl.mo); };
        pl.group = WI;
        int cps = std::max(1, plan_ctas_per_sm(pl));
        // Measured on GB300 (tuner sweeps): one warp row per tile and no split are best
        // whenever the tiles alone cover the grid; otherwise two warp rows per tile
        // (more only when q is too short to split), then split q until about two
        // items per CTA.
        const uint64_t grid_full = (uint64_t)sms * cps;
        // tiles that keep the HBM system busy: a full grid, or 4 CTAs per SM for the
        // narrow-load kernels that fit more (fp32 strided: 6 per SM; rows of 645 with
        // 813 tiles, one warp row and no split: 168-180 us against 191-205 us)
        uint64_t fill = std::min<uint64_t>(grid_full, (uint64_t)sms * 4);
        if (force_group <= 0 && tiles_for(1) < fill) {
            WI = 2;
            while (WI < 8 && cn.nq < 64 && tiles_for(WI) < grid_full && cn.nq >= (uint64_t)WI * 2 * 4) WI *= 2;
            pl.group = WI;
            cps = std::max(1, plan_ctas_per_sm(pl));
            fill = std::min<uint64_t>((uint64_t)sms * cps, (uint64_t)sms * 4);
        }
        const uint64_t want = 2 * (uint64_t)sms * cps;
        const uint64_t tiles = tiles_for(WI);
        uint64_t nseg = cdiv(cn.nq, bmax);
        if (force_split > 0) {
            nseg = std::max<uint64_t>(nseg, (uint64_t)force_split);
            if ((uint64_t)force_split < cdiv(cn.nq, bmax))
                return fail(TLIBG_ERR_ARGUMENT, "tlibg: forced split leaves a segment longer than the staged b buffer");
        } else if (tiles < fill && tiles * nseg < want) {
            const uint64_t min_len = (uint64_t)WI * 4 * 4;
            nseg = std::max<uint64_t>(nseg, std::min<uint64_t>(cdiv(want, tiles), std::max<uint64_t>(1, cn.nq / min_len)));
        }
        nseg = std::max<uint64_t>(1, std::min<uint64_t>(nseg, cn.nq));
        uint64_t seg_len = cdiv(cn.nq, nseg);
        nseg = cdiv(cn.nq, seg_len);
        pl.split = (int)nseg;
        pl.seg_len = seg_len;
        pl.items = tiles * nseg;
        const uint64_t max_grid = (uint64_t)sms * cps;
        uint64_t grid = std::min<uint64_t>(max_grid, pl.items);
        pl.items_per_cta = cdiv(pl.items, grid);
        pl.grid = (int)cdiv(pl.items, pl.items_per_cta);
    }
    pl.f64_combine = (dtype != F64) && pl.split > 1 && cn.nq > (uint64_t(1) << 20);
    pl.smem = plan_smem_bytes(pl);
    *out = pl;
    return TLIBG_OK;
}

// --------------------------------------------------------------------------
// per-(device, stream) scratch for split partials (grow-only)
// --------------------------------------------------------------------------
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};
std::mutex g_scratch_mu;
std::map<std::pair<int, uintptr_t>, Scratch> g_scratch;

int get_scratch(cudaStream_t stream, size_t bytes, void** out)
{
    if (bytes == 0) {
        *out = nullptr;
        return TLIBG_OK;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    Scratch& s = g_scratch[{dev, reinterpret_cast<uintptr_t>(stream)}];
    if (s.bytes < bytes) {
        if (s.ptr) {
            // the previous buffer may still be read by work queued on this stream
            cudaStreamSynchronize(stream);
            cudaFree(s.ptr);
            s.ptr = nullptr;
            s.bytes = 0;
        }
        size_t want = std::max(bytes, (size_t)1 << 20);
        cudaError_t e = device_malloc(&s.ptr, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(TLIBG_ERR_NOMEM, std::string("tlibg: cannot allocate split scratch: ") + cudaGetErrorString(e));
        }
        s.bytes = want;
    }
    *out = s.ptr;
    return TLIBG_OK;
}

// Pageable host memory is not addressable by the kernels: refuse it up front
// (pinned host memory and managed memory are device-accessible and pass).
int check_device_pointers(const void* a, const void* b, const void* c)
{
    for (const void* p : {a, b, c}) {
        cudaPointerAttributes at{};
        const cudaError_t e = cudaPointerGetAttributes(&at, p);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_fail(e, "cudaPointerGetAttributes");
        }
        if (at.type == cudaMemoryTypeUnregistered)
            return fail(TLIBG_ERR_ARGUMENT, "tlibg: a, b and c must be device-accessible pointers "
                                            "(host buffers: tlibg_ttv_host)");
    }
    return TLIBG_OK;
}

// Every kernel addresses A, b and C per element (and wider): pointers must
// be aligned to their element types, as a C or C++ caller's own are.
int check_elem_align(int dtype, const void* a, const void* b, const void* c)
{
    if (!aligned(a, elem_size_a(dtype)) || !aligned(b, elem_size_t(dtype)) || !aligned(c, elem_size_t(dtype)))
        return fail(TLIBG_ERR_UNSUPPORTED, "tlibg: a, b and c must be aligned to their element sizes");
    return TLIBG_OK;
}

int run_device(int dtype, size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
               const size_t* pia, const void* b, const size_t* nb, void* c, const size_t* nc,
               const size_t* wc, const size_t* pic, const tlibg_options* opt, cudaStream_t stream)
{
    NvtxRange nvtx("tlibg_ttv");
    Canon cn;
    int st = analyse(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, &cn);
    if (st) return st;
    st = check_elem_align(dtype, a, b, c);
    if (st) return st;
    DevInfo d = dev_info();
    if (!d.ok) return fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    st = check_device_pointers(a, b, c);
    if (st) return st;
    Plan pl;
    st = make_plan(dtype, cn, a, b, opt, d.sms, &pl);
    if (st) return st;
    void* part = nullptr;
    st = get_scratch(stream, partial_bytes(pl), &part);
    if (st) return st;
    uint64_t launches = 0;
    cudaError_t e = launch_plan(pl, a, b, c, part, stream, &launches);
    g_launches += launches;
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    if (opt && opt->sync) {
        e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
        unsigned int derr = read_and_clear_device_error();
        if (derr) return fail(TLIBG_ERR_TIMEOUT, "tlibg: a bounded device wait expired; results are invalid");
    }
    return ok();
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int tlibg_ttv_f32(size_t q, size_t p, const float* a, const size_t* na, const size_t* wa,
                  const size_t* pia, const float* b, const size_t* nb, float* c, const size_t* nc,
                  const size_t* wc, const size_t* pic, void* stream)
{
    return run_device(F32, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, nullptr,
                      static_cast<cudaStream_t>(stream));
}

int tlibg_ttv_f64(size_t q, size_t p, const double* a, const size_t* na, const size_t* wa,
                  const size_t* pia, const double* b, const size_t* nb, double* c, const size_t* nc,
                  const size_t* wc, const size_t* pic, void* stream)
{
    return run_device(F64, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, nullptr,
                      static_cast<cudaStream_t>(stream));
}

int tlibg_ttv_bf16a_f32(size_t q, size_t p, const uint16_t* a, const size_t* na, const size_t* wa,
                        const size_t* pia, const float* b, const size_t* nb, float* c,
                        const size_t* nc, const size_t* wc, const size_t* pic, void* stream)
{
    return run_device(BF16A, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, nullptr,
                      static_cast<cudaStream_t>(stream));
}

int tlibg_ttv_ex(int dtype, size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                 const size_t* pia, const void* b, const size_t* nb, void* c, const size_t* nc,
                 const size_t* wc, const size_t* pic, const tlibg_options* opt, void* stream)
{
    if (dtype != F32 && dtype != F64 && dtype != BF16A)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: unknown element type");
    return run_device(dtype, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, opt,
                      static_cast<cudaStream_t>(stream));
}

int tlibg_validate(size_t q, size_t p, const size_t* na, const size_t* wa, const size_t* pia,
                   const size_t* nb, const size_t* nc, const size_t* wc, const size_t* pic)
{
    // the data pointers only take part in null checks: stand-ins let the
    // metadata checks run in the reference's order without touching memory
    static const char stand_in = 0;
    Canon cn;
    const int st = analyse(q, p, &stand_in, na, wa, pia, &stand_in, nb, &stand_in, nc, wc, pic, &cn);
    return st ? st : ok();
}

int tlibg_selftest_bounded_wait(void* stream)
{
    DevInfo d = dev_info();
    if (!d.ok) return fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_wait_probe(st, 1u << 14);
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    g_launches += 1;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "stream synchronize");
    if (read_and_clear_device_error())
        return fail(TLIBG_ERR_TIMEOUT, "tlibg: a bounded device wait expired; results are invalid");
    return ok();
}

int tlibg_pointer_location(const void* p)
{
    if (!p) return -1;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return 0;   // no device: every pointer is a host pointer
    }
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return 1;
    return 0;
}

int tlibg_plan(int dtype, size_t q, size_t p, const size_t* na, const size_t* pia,
               const tlibg_options* opt, tlibg_plan_info* out)
{
    if (!out) return fail(TLIBG_ERR_ARGUMENT, "tlibg: plan output is null");
    if (dtype != F32 && dtype != F64 && dtype != BF16A)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: unknown element type");
    if (p == 0) return fail(TLIBG_ERR_ARGUMENT, MSG[1]);
    if (q == 0 || q > p) return fail(TLIBG_ERR_ARGUMENT, MSG[2]);
    if (!na || !pia) return fail(TLIBG_ERR_ARGUMENT, "tlibg: shape and layout are required");
    if (!valid_shape(na, p)) return fail(TLIBG_ERR_ARGUMENT, MSG[14]);
    if (!valid_layout(pia, p)) return fail(TLIBG_ERR_ARGUMENT, MSG[16]);
    Canon cn;
    size_t k = 0;
    while (pia[k] != q) ++k;
    for (size_t r = 0; r < k; ++r) cn.P *= na[pia[r] - 1];
    for (size_t r = k + 1; r < p; ++r) cn.S *= na[pia[r] - 1];
    cn.nq = na[q - 1];
    DevInfo d = dev_info();
    const int sms = d.ok ? d.sms : PLAN_SMS_WITHOUT_DEVICE;
    Plan pl;
    // plan for 256-byte aligned device buffers (what cudaMalloc returns)
    static const uint4 probe_a[1] = {};
    int st = make_plan(dtype, cn, probe_a, probe_a, opt, sms, &pl);
    if (st) return st;
    out->P = pl.P;
    out->nq = pl.nq;
    out->S = pl.S;
    out->kind = pl.kind;
    out->group = pl.group;
    out->vec = pl.vec;
    out->split = pl.split;
    out->accumulate = pl.kahan ? TLIBG_ACC_COMPENSATED : TLIBG_ACC_PLAIN;
    out->grid = pl.grid;
    out->block = pl.kind == KIND_STREAM ? STREAM_CONSUMERS + 32
                 : (pl.kind == KIND_ROW_TILE ? ROWT_THREADS : (pl.kind == KIND_COL_BULK ? CB_THREADS : BLOCK));
    return ok();
}

// ---------------------------------------------------------------------------
// general strides (extension; the drop-in calls keep the dense-only rule)
// ---------------------------------------------------------------------------
int tlibg_ttv_strided(int dtype, size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                      const size_t* pia, const void* b, const size_t* nb, size_t wb, void* c, const size_t* nc,
                      const size_t* wc, const size_t* pic, void* stream)
{
    NvtxRange nvtx("tlibg_ttv_strided");
    if (dtype != F32 && dtype != F64)
        return fail(dtype == BF16A ? TLIBG_ERR_UNSUPPORTED : TLIBG_ERR_ARGUMENT,
                    dtype == BF16A ? "tlibg_ttv_strided: fp32 and fp64 only" : "tlibg: unknown element type");
    // the reference's checks and messages (shape, layout, monotonic strides, C's metadata)
    const int code = check_call(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
    if (code) return fail(TLIBG_ERR_ARGUMENT, MSG[code]);
    if (p - 1 > (size_t)GS_MAX_MODES) return fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttv_strided: at most 17 modes");
    if (wb == 0) return fail(TLIBG_ERR_ARGUMENT, "tlibg_ttv_strided: b's stride must be at least 1");
    // natural meaning: every output its own element of C (no two outputs share an
    // address), every offset within 2^62 elements
    {
        std::vector<std::pair<size_t, size_t>> sw;   // (stride, extent) of C's modes with extent > 1
        for (size_t r = 0; r + 1 < p; ++r)
            if (nc[r] > 1) sw.push_back({wc[r], nc[r]});
        std::sort(sw.begin(), sw.end());
        uint64_t span = 1;
        for (auto& e : sw) {
            if (e.first < span)
                return fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttv_strided: C's strides make two outputs share an "
                                                   "element");
            uint64_t t;
            if (mul_overflows(e.first, e.second, &t)) return fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttv_strided: "
                                                                                         "offsets exceed 2^62");
            span = t;
        }
        uint64_t amax = 0;
        for (size_t r = 0; r < p; ++r) {
            uint64_t t;
            if (mul_overflows(na[r] - 1, wa[r], &t) || (amax += t) > (uint64_t(1) << 62))
                return fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttv_strided: offsets exceed 2^62");
        }
        uint64_t t;
        if (mul_overflows(na[q - 1] - 1, wb, &t)) return fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttv_strided: "
                                                                                     "offsets exceed 2^62");
    }
    if (int st = check_elem_align(dtype, a, b, c)) return st;
    if (!dev_info().ok) return fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    if (int st = check_device_pointers(a, b, c)) return st;

    // modes other than q, A-stride order; C's mode r (0-based) is A's mode r or r + 1
    GSArgs k{};
    std::vector<std::tuple<size_t, size_t, size_t>> modes;   // (wa, extent, wc)
    for (size_t m = 0; m < p; ++m) {
        if (m == q - 1) continue;
        const size_t cm = m < q - 1 ? m : m - 1;
        if (na[m] > 1) modes.emplace_back(wa[m], na[m], wc[cm]);
    }
    std::sort(modes.begin(), modes.end());
    k.nm = (int)modes.size();
    k.outputs = 1;
    for (int r = 0; r < k.nm; ++r) {
        k.wa[r] = std::get<0>(modes[r]);
        k.ext[r] = std::get<1>(modes[r]);
        k.wc[r] = std::get<2>(modes[r]);
        k.outputs *= k.ext[r];
    }
    k.a = a;
    k.b = b;
    k.c = c;
    k.nq = na[q - 1];
    k.waq = na[q - 1] > 1 ? wa[q - 1] : 0;
    k.wb = wb;
    const bool row = k.nm == 0 || (k.nq > 1 && k.waq <= k.wa[0]);
    k.group = (uint32_t)std::max(1, std::min(32, pow2_floor(std::max<uint64_t>(1, k.nq / 16))));
    const int sms = dev_info().sms;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // 16-byte forms where the view allows them
    const uint64_t V = 16 / (dtype == F64 ? 8 : 4);
    bool others_on_grid = (reinterpret_cast<uintptr_t>(a) % 16) == 0;
    for (int r = 0; r < k.nm; ++r) others_on_grid = others_on_grid && k.wa[r] % V == 0;
    const bool row_vec = row && k.waq == 1 && k.nq % V == 0 && wb == 1 &&
                         (reinterpret_cast<uintptr_t>(b) % 16) == 0 && others_on_grid;
    bool col_vec = !row && k.nm > 0 && k.wa[0] == 1 && k.ext[0] % V == 0 &&
                   (reinterpret_cast<uintptr_t>(a) % 16) == 0 && k.waq % V == 0;
    for (int r = 1; r < k.nm; ++r) col_vec = col_vec && k.wa[r] % V == 0;
    // one thread per V outputs only while the outputs alone still fill the GPU (the
    // column forms take no split of n_q): measured on 2^26-element padded views,
    // 131072 outputs over 512 rows ran 1.8 TB/s with V per thread, 4.1 with one
    col_vec = col_vec && k.outputs / V >= (uint64_t)sms * 1024;
    const uint64_t threads = row ? k.outputs * k.group : (col_vec ? k.outputs / V : k.outputs);
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 8, (threads + 255) / 256));
    if (dtype == F64) {
        if (row_vec) gs_row_vec_kernel<double><<<grid, 256, 0, st>>>(k);
        else if (row) gs_row_kernel<double><<<grid, 256, 0, st>>>(k);
        else if (col_vec) gs_col_vec_kernel<double><<<grid, 256, 0, st>>>(k);
        else gs_col_kernel<double><<<grid, 256, 0, st>>>(k);
    } else {
        if (row_vec) gs_row_vec_kernel<float><<<grid, 256, 0, st>>>(k);
        else if (row) gs_row_kernel<float><<<grid, 256, 0, st>>>(k);
        else if (col_vec) gs_col_vec_kernel<float><<<grid, 256, 0, st>>>(k);
        else gs_col_kernel<float><<<grid, 256, 0, st>>>(k);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    g_launches += 1;
    return ok();
}

// ---------------------------------------------------------------------------
// host-buffer path: chunked copies overlapped with the kernels
// ---------------------------------------------------------------------------
// Copy of n16 16-byte blocks from page-locked host memory (through its device
// address) to device memory: four loads in flight per thread, each warp load one
// 512-byte run.
__global__ void __launch_bounds__(256) host_stage_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src,
                                                         uint64_t n16)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = src[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u) dst[i + u * stride] = v[u];
    }
    for (; i < n16; i += stride) dst[i] = src[i];
}

// Bytes of A per staged chunk (MB), and the in-place read rule (-1: by plan, as
// described below; 0: always staged; 1: in place whenever A is page-locked).
#ifndef TLIBG_HOST_CHUNK_MB
#define TLIBG_HOST_CHUNK_MB 64
#endif
#ifndef TLIBG_HOST_DIRECT
#define TLIBG_HOST_DIRECT -1
#endif

int tlibg_ttv_host(int dtype, size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                   const size_t* pia, const void* b, const size_t* nb, void* c, const size_t* nc,
                   const size_t* wc, const size_t* pic, const tlibg_options* opt)
{
    if (dtype != F32 && dtype != F64 && dtype != BF16A)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg: unknown element type");
    NvtxRange nvtx("tlibg_ttv_host");
    Canon cn;
    int st = analyse(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, &cn);
    if (st) return st;
    DevInfo d = dev_info();
    if (!d.ok) return fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");

    const size_t ea = elem_size_a(dtype), et = elem_size_t(dtype);
    // chunk along the suffix S (independent panels); one chunk when S == 1
    const uint64_t panel = cn.nq * cn.P;                     // elements of A per panel
    const uint64_t chunk_bytes_target = (uint64_t)TLIBG_HOST_CHUNK_MB << 20;
    uint64_t spc = std::max<uint64_t>(1, chunk_bytes_target / std::max<uint64_t>(1, panel * ea));
    spc = std::min<uint64_t>(spc, cn.S);
    const uint64_t nchunks = cdiv(cn.S, spc);

    struct HostCtx {
        cudaStream_t comp = nullptr, copy = nullptr;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        cudaEvent_t done[2] = {nullptr, nullptr};
        void* abuf[2] = {nullptr, nullptr};
        size_t abytes = 0;
        void* bbuf = nullptr;
        size_t bbytes = 0;
        void* cbuf = nullptr;
        size_t cbytes = 0;
    };
    static std::mutex mu;
    static std::map<int, HostCtx> ctxs;
    std::lock_guard<std::mutex> lk(mu);
    int dev = 0;
    cudaGetDevice(&dev);
    HostCtx& hc = ctxs[dev];
    cudaError_t e;
    if (!hc.comp) {
        if ((e = cudaStreamCreateWithFlags(&hc.comp, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream create");
        if ((e = cudaStreamCreateWithFlags(&hc.copy, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream create");
        for (int i = 0; i < 2; ++i) {
            cudaEventCreateWithFlags(&hc.ev[i], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&hc.done[i], cudaEventDisableTiming);
        }
    }
    const size_t need_a = (size_t)(spc * panel * ea) + 32;   // + the 16-byte cover of a chunk
    const size_t need_b = (size_t)(cn.nq * et);
    const size_t need_c = (size_t)(cn.S * cn.P * et);
    auto grow = [&](void** p_, size_t* have, size_t need) -> int {
        if (*have >= need) return TLIBG_OK;
        if (*p_) cudaFree(*p_);
        *p_ = nullptr;
        *have = 0;
        cudaError_t ee = device_malloc(p_, need);
        if (ee != cudaSuccess) {
            cudaGetLastError();
            return fail(TLIBG_ERR_NOMEM, "tlibg: cannot allocate device staging buffers");
        }
        *have = need;
        return TLIBG_OK;
    };
    if ((st = grow(&hc.bbuf, &hc.bbytes, need_b))) return st;
    if ((st = grow(&hc.cbuf, &hc.cbytes, need_c))) return st;

    // Page-locked A whose plan reads 512-byte runs per warp load (column tiles with
    // 16-byte loads, rows taken by a whole warp): the kernels read it in place over
    // the host link (one pass, no staging copy; on GB300 such reads move
    // page-locked memory as fast as the copy engines do).  Every other plan (short
    // rows, whose lane groups issue one short run per row, and scalar loads) goes
    // through the staged path below: chunks copied into device memory by the SMs
    // (512-byte runs per warp load again) overlapped with the device kernels
    // (measured over the symmetric sweep: rows of 16-25 elements 123-149 GB/s read
    // in place against the 211 GB/s link; copy-engine staging of the same chunks
    // varied from 27 to 200 GB/s between runs).  The bulk copies of the streamed,
    // row-tile and TMA-staged column kernels are kept to device memory.
    cudaPointerAttributes at{};
    const bool a_pinned = cudaPointerGetAttributes(&at, a) == cudaSuccess && at.type == cudaMemoryTypeHost &&
                          at.devicePointer != nullptr;
    cudaGetLastError();
    cudaPointerAttributes atc{};
    // Page-locked C is written in place by the kernels only where that pays: column
    // forms (each warp stores contiguous runs) with C at least 1/16 of A, whose copy
    // after the kernels would cost time.  Row forms store one short run per row
    // group, and such scattered stores over the host link measured from 27 to
    // 200 GB/s depending on where the buffer sits; their C, like the smaller C of
    // longer contractions, goes to device memory and back in one copy.
    const bool c_pinned = cudaPointerGetAttributes(&atc, c) == cudaSuccess && atc.type == cudaMemoryTypeHost &&
                          atc.devicePointer != nullptr && cn.P > 1 && cn.nq <= 16;   // C >= A / 16
    cudaGetLastError();
    bool direct = false;
    if (a_pinned) {
        tlibg_options o2{TLIBG_ACC_COMPENSATED, -1, 0, 0, 0, 0};
        if (opt) o2 = *opt;
        if (o2.kind == KIND_STREAM || o2.kind == KIND_ROW_TILE || o2.kind == KIND_COL_BULK) o2.kind = -1;
        Plan probe_pl;
        if ((st = make_plan(dtype, cn, at.devicePointer, hc.bbuf, &o2, d.sms, &probe_pl))) return st;
        // a warp's 16-byte loads cover one 512-byte run: column tiles, thin prefixes of
        // at least 512 bytes, rows taken by a whole warp
        const bool v16 = (size_t)probe_pl.vec * ea == 16;
        direct = v16 && (probe_pl.kind == KIND_COL ||
                         (probe_pl.kind == KIND_COL_THIN && cn.P * ea >= 512) ||
                         (probe_pl.kind == KIND_ROW && probe_pl.group == 32 && probe_pl.rows_m == 0));
        if (TLIBG_HOST_DIRECT >= 0) direct = TLIBG_HOST_DIRECT == 1;
    }
    if (a_pinned && direct) {
        if ((e = cudaMemcpyAsync(hc.bbuf, b, need_b, cudaMemcpyHostToDevice, hc.comp)) != cudaSuccess)
            return cuda_fail(e, "copy of b");
        // page-locked C too: the kernels store C in place over the link while they
        // read A (the link carries both directions at once), no copy after them
        void* cdst = c_pinned ? atc.devicePointer : hc.cbuf;
        tlibg_options o2{TLIBG_ACC_COMPENSATED, -1, 0, 0, 0, 0};
        if (opt) o2 = *opt;
        if (o2.kind == KIND_STREAM || o2.kind == KIND_ROW_TILE || o2.kind == KIND_COL_BULK) o2.kind = -1;
        Plan pl;
        if ((st = make_plan(dtype, cn, at.devicePointer, hc.bbuf, &o2, d.sms, &pl))) return st;
        if (pl.kind == KIND_STREAM || pl.kind == KIND_ROW_TILE || pl.kind == KIND_COL_BULK) {
            o2.kind = cn.P == 1 ? KIND_ROW : KIND_COL;
            if ((st = make_plan(dtype, cn, at.devicePointer, hc.bbuf, &o2, d.sms, &pl))) return st;
        }
        void* part = nullptr;
        if ((st = get_scratch(hc.comp, partial_bytes(pl), &part))) return st;
        uint64_t launches = 0;
        e = launch_plan(pl, at.devicePointer, hc.bbuf, cdst, part, hc.comp, &launches);
        g_launches += launches;
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        if (!c_pinned && (e = cudaMemcpyAsync(c, hc.cbuf, need_c, cudaMemcpyDeviceToHost, hc.comp)) != cudaSuccess)
            return cuda_fail(e, "copy of C");
        if ((e = cudaStreamSynchronize(hc.comp)) != cudaSuccess) return cuda_fail(e, "stream synchronize");
        if (read_and_clear_device_error())
            return fail(TLIBG_ERR_TIMEOUT, "tlibg: a bounded device wait expired; results are invalid");
        return ok();
    }

    // staged path: two chunk buffers in device memory (only this path needs them)
    if (hc.abytes < need_a) {
        cudaStreamSynchronize(hc.comp);
        cudaStreamSynchronize(hc.copy);
        for (int i = 0; i < 2; ++i) {
            if (hc.abuf[i]) cudaFree(hc.abuf[i]);
            hc.abuf[i] = nullptr;
        }
        hc.abytes = 0;
        for (int i = 0; i < 2; ++i)
            if (device_malloc(&hc.abuf[i], need_a) != cudaSuccess) {
                cudaGetLastError();
                return fail(TLIBG_ERR_NOMEM, "tlibg: cannot allocate device staging buffers");
            }
        hc.abytes = need_a;
    }
    if ((e = cudaMemcpyAsync(hc.bbuf, b, need_b, cudaMemcpyHostToDevice, hc.copy)) != cudaSuccess)
        return cuda_fail(e, "copy of b");
    uint64_t launches = 0;
    for (uint64_t k = 0; k < nchunks; ++k) {
        const int slot = (int)(k & 1);
        const uint64_t s0 = k * spc;
        const uint64_t sn = std::min<uint64_t>(spc, cn.S - s0);
        // the copy into this slot must wait until the kernels that read it are done
        if (k >= 2) cudaStreamWaitEvent(hc.copy, hc.done[slot], 0);
        const char* src = static_cast<const char*>(a) + s0 * panel * ea;
        const size_t len = (size_t)(sn * panel * ea);
        char* adev = static_cast<char*>(hc.abuf[slot]);
        if (a_pinned) {
            // page-locked A: the SMs copy the chunk's 16-byte-aligned cover (one 512-byte
            // run per warp load, the kind of read that keeps the host link full), and the
            // kernels read the chunk at its own offset in the cover
            const char* hsrc = static_cast<const char*>(at.devicePointer) + s0 * panel * ea;
            const uintptr_t lo = reinterpret_cast<uintptr_t>(hsrc) & ~uintptr_t(15);
            const uintptr_t hi = (reinterpret_cast<uintptr_t>(hsrc) + len + 15) & ~uintptr_t(15);
            const uint64_t n16 = (hi - lo) / 16;
            const int grid = (int)std::min<uint64_t>((uint64_t)d.sms * 2, std::max<uint64_t>(1, n16 / 1024));
            host_stage_kernel<<<grid, 256, 0, hc.copy>>>(reinterpret_cast<uint4*>(adev),
                                                         reinterpret_cast<const uint4*>(lo), n16);
            if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "copy of A");
            ++launches;
            adev += reinterpret_cast<uintptr_t>(hsrc) - lo;
        } else if ((e = cudaMemcpyAsync(adev, src, len, cudaMemcpyHostToDevice, hc.copy)) != cudaSuccess) {
            return cuda_fail(e, "copy of A");
        }
        cudaEventRecord(hc.ev[slot], hc.copy);
        cudaStreamWaitEvent(hc.comp, hc.ev[slot], 0);
        Canon ck = cn;
        ck.S = sn;
        Plan pl;
        if ((st = make_plan(dtype, ck, adev, hc.bbuf, opt, d.sms, &pl))) return st;
        void* part = nullptr;
        if ((st = get_scratch(hc.comp, partial_bytes(pl), &part))) return st;
        // page-locked C: each chunk's kernels store their part of C in place
        char* cdst = static_cast<char*>(c_pinned ? atc.devicePointer : hc.cbuf) + s0 * cn.P * et;
        e = launch_plan(pl, adev, hc.bbuf, cdst, part, hc.comp, &launches);
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        cudaEventRecord(hc.done[slot], hc.comp);
    }
    g_launches += launches;
    if (!c_pinned && (e = cudaMemcpyAsync(c, hc.cbuf, need_c, cudaMemcpyDeviceToHost, hc.comp)) != cudaSuccess)
        return cuda_fail(e, "copy of C");
    if ((e = cudaStreamSynchronize(hc.comp)) != cudaSuccess) return cuda_fail(e, "stream synchronize");
    unsigned int derr = read_and_clear_device_error();
    if (derr) return fail(TLIBG_ERR_TIMEOUT, "tlibg: a bounded device wait expired; results are invalid");
    return ok();
}

// ---------------------------------------------------------------------------
// metadata helpers
// ---------------------------------------------------------------------------
int tlibg_output_shape(const size_t* na, size_t p, size_t q, size_t* nc)
{
    if (!na || !valid_shape(na, p))
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::generate_output_shape(): input shape is not valid.");
    if (q == 0 || q > p)
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::generate_output_shape(): constraction mode q "
                                        "should be greater than 0 and less than or equal to the tensor order.");
    size_t o = 0;
    for (size_t r = 0; r < p; ++r)
        if (r != q - 1) nc[o++] = na[r];
    return ok();
}

int tlibg_output_layout(const size_t* pia, size_t p, size_t q, size_t* pic)
{
    if (!pia || !valid_layout(pia, p))
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::generate_output_layout(): input layout is not valid.");
    if (q == 0 || q > p)
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::generate_output_layout(): constraction mode q "
                                        "should be greater than 0 and less than or equal to the tensor order.");
    size_t o = 0;
    for (size_t r = 0; r < p; ++r) {
        if (pia[r] == q) continue;
        pic[o++] = pia[r] > q ? pia[r] - 1 : pia[r];
    }
    return ok();
}

int tlibg_strides(const size_t* n, const size_t* pi, size_t p, size_t* w)
{
    if (!n || !valid_shape(n, p))
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::compute_strides(): input shape is not valid.");
    if (!pi || !valid_layout(pi, p))
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::compute_strides(): input layout is not valid.");
    dense_strides(n, pi, p, w);
    return ok();
}

int tlibg_k_order_layout(size_t p, size_t k, size_t* pi)
{
    if (p == 0)
        return fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::compute_k_order: range provided by begin and end not correct!");
    if (k == 0) k = p;
    const size_t m = std::min(k, p);
    size_t r = 0;
    for (size_t v = m; r < m; --v, ++r) pi[r] = v;
    for (size_t v = m + 1; r < p; ++v, ++r) pi[r] = v;
    return ok();
}

size_t tlibg_inverse_mode(const size_t* pi, size_t p, size_t mode)
{
    if (!pi || !valid_layout(pi, p)) {
        fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::inverse_mode(): input layout is not valid.");
        return 0;
    }
    if (mode == 0 || mode > p) {
        fail(TLIBG_ERR_ARGUMENT, "Error in tlib::detail::inverse_mode(): mode should be one-based and equal "
                                 "to or less than layout size.");
        return 0;
    }
    for (size_t r = 0; r < p; ++r)
        if (pi[r] == mode) {
            ok();
            return r + 1;
        }
    return 0;
}

int tlibg_plan_hint(int dtype, uint64_t P, uint64_t nq, uint64_t S, const tlibg_options* opt)
{
    std::lock_guard<std::mutex> lk(g_hint_mu);
    if (!opt) {
        if (P == 0 && nq == 0 && S == 0) g_hints.clear();
        else g_hints.erase(std::make_tuple(dtype, P, nq, S));
        return ok();
    }
    if (dtype != F32 && dtype != F64 && dtype != BF16A)
        return fail(TLIBG_ERR_ARGUMENT, "tlibg_plan_hint: unknown element type");
    g_hints[std::make_tuple(dtype, P, nq, S)] = *opt;
    return ok();
}

size_t tlibg_last_error(char* buf, size_t len)
{
    if (buf && len) {
        size_t n = std::min(len - 1, t_last_error.size());
        std::memcpy(buf, t_last_error.data(), n);
        buf[n] = 0;
    }
    return t_last_error.size();
}

int tlibg_device_error(void)
{
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (int)read_and_clear_device_error();
}

uint64_t tlibg_launch_count(void) { return g_launches.load(); }

uint64_t tlibg_device_alloc_count(void) { return g_device_allocs.load(); }

const char* tlibg_version(void) { return "tlibg 0.1 (sm_103a)"; }

}  // extern "C"

// ============================================================================
// Allocation-free entry point
// ============================================================================
// Some callers cannot let this library allocate device memory: frameworks
// whose caching allocator owns (and accounts for) every device byte, memory-
// budgeted or multi-tenant processes, and latency-critical loops where the
// implicit device synchronisation of cudaMalloc / cudaFree is not acceptable.
// tlibg_ttv_f32_noalloc serves them: the only device memory it uses besides
// the caller's a, b and c is the split-reduction scratch below, a fixed array
// compiled into the library.  Every device that loads the library holds it
// (TLIBG_NOALLOC_SCRATCH_BYTES) until the process exits.
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TLIBG_NOALLOC_SCRATCH_BYTES];

// cuCtxGetCurrent through the runtime's driver entry point (the library does
// not link the driver library itself).
typedef int (*CtxGetCurrentFn)(void**);

CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    return fn;
}

// Device address of g_noalloc_scratch, resolved once per (device, context)
// with that device current.  In host code the array's name is only a
// host-side stand-in for the symbol, never a device address, so kernels get
// this pointer.  The context is part of the key: after cudaDeviceReset (or any
// new primary context) the module is loaded again and the array may live at
// another address.
int noalloc_scratch(void** out)
{
    static std::mutex mu;
    static std::map<std::pair<int, uintptr_t>, void*> addr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    // cudaSetDevice makes the device's primary context current (initialising it
    // if need be), so the context read below is the one the kernels run in
    if ((e = cudaSetDevice(dev)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    void* ctx = nullptr;
    if (CtxGetCurrentFn f = ctx_get_current()) f(&ctx);
    const auto key = std::make_pair(dev, reinterpret_cast<uintptr_t>(ctx));
    std::lock_guard<std::mutex> lk(mu);
    auto it = addr.find(key);
    if (it != addr.end()) {
        *out = it->second;
        return TLIBG_OK;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
        return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress");
    addr[key] = p;
    *out = p;
    return TLIBG_OK;
}

}  // namespace

extern "C" int tlibg_ttv_f32_noalloc(size_t q, size_t p, const float* a, const size_t* na,
                                     const size_t* wa, const size_t* pia, const float* b,
                                     const size_t* nb, float* c, const size_t* nc,
                                     const size_t* wc, const size_t* pic, void* stream)
{
    NvtxRange nvtx("tlibg_ttv_f32_noalloc");
    Canon cn;
    int st = analyse(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, &cn);
    if (st) return st;
    st = check_elem_align(F32, a, b, c);
    if (st) return st;
    DevInfo d = dev_info();
    if (!d.ok) return fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    st = check_device_pointers(a, b, c);
    if (st) return st;
    const size_t limit = (size_t)TLIBG_NOALLOC_SCRATCH_BYTES;
    Plan pl;
    st = make_plan(F32, cn, a, b, nullptr, d.sms, &pl);
    if (st) return st;
    size_t need = partial_bytes(pl);
    if (need > limit) {
        // The planner's split needs more scratch than the array holds: plan again
        // with the split capped at the most segments whose partials fit (the
        // kernels' own lower bound on segments still applies), then without a
        // split; refuse only if neither plan fits.
        const size_t per_seg = (size_t)(cn.S * cn.P) * 2 * sizeof(float);
        const size_t cap = per_seg ? limit / per_seg : 0;
        bool found = false;
        for (size_t k : {cap, (size_t)1}) {
            if (k < 1) continue;
            tlibg_options o{TLIBG_ACC_COMPENSATED, -1, 0, 0, (int)std::min<size_t>(k, 1u << 30), 0};
            Plan alt;
            if (make_plan_inner(F32, cn, a, b, &o, d.sms, &alt) != TLIBG_OK) continue;
            if (partial_bytes(alt) <= limit) {
                pl = alt;
                need = partial_bytes(alt);
                found = true;
                break;
            }
        }
        if (!found)
            return fail(TLIBG_ERR_UNSUPPORTED,
                        "tlibg_ttv_f32_noalloc: this problem's split reduction needs " + std::to_string(need) +
                            " bytes of scratch, more than the fixed " + std::to_string(limit) +
                            "-byte buffer; use tlibg_ttv_f32");
    }
    void* part = nullptr;
    if (need) {
        st = noalloc_scratch(&part);
        if (st) return st;
    }
    // Nothing in the scratch needs to start at zero: the main kernel writes
    // every partial slot the combine kernel then reads, within this call.
    uint64_t launches = 0;
    cudaError_t e = launch_plan(pl, a, b, c, part, static_cast<cudaStream_t>(stream), &launches);
    g_launches += launches;
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return ok();
}

// ============================================================================
// internal interface for the other translation units (ttv_internal.h)
// ============================================================================
namespace tlibg {

int internal_analyse(size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                     const size_t* pia, const void* b, const size_t* nb, const void* c,
                     const size_t* nc, const size_t* wc, const size_t* pic, CanonView* out)
{
    Canon cn;
    const int st = analyse(q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, &cn);
    if (st) return st;
    out->P = cn.P;
    out->nq = cn.nq;
    out->S = cn.S;
    out->ref_case = cn.ref_case;
    return TLIBG_OK;
}

int internal_plan(int dtype, const CanonView& cv, const void* a, const void* b,
                  const tlibg_options* opt, int sms, Plan* out)
{
    Canon cn;
    cn.P = cv.P;
    cn.nq = cv.nq;
    cn.S = cv.S;
    cn.ref_case = cv.ref_case;
    return make_plan(dtype, cn, a, b, opt, sms, out);
}

int internal_sms()
{
    DevInfo d = dev_info();
    return d.ok ? d.sms : 0;
}

int internal_fail(int code, const std::string& msg) { return fail(code, msg); }
int internal_ok() { return ok(); }
int internal_check_device_pointers(const void* a, const void* b, const void* c)
{
    return check_device_pointers(a, b, c);
}
int internal_cuda_fail(cudaError_t e, const char* where) { return cuda_fail(e, where); }
cudaError_t internal_malloc(void** p, size_t bytes) { return device_malloc(p, bytes); }
int internal_scratch(cudaStream_t stream, size_t bytes, void** out) { return get_scratch(stream, bytes, out); }
void internal_count_launches(uint64_t n) { g_launches += n; }

}  // namespace tlibg
