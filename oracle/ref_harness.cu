// ref_harness.cu — runs the reference's own compiled kernels.  TEST INFRASTRUCTURE ONLY.
//
// The reference (ZZPHUB/tmp_sph: src/ and the snapshots opt_src_v0..v4) is CUDA C++; its
// kernels are compiled here from its own sources into fatbins (oracle/ref_build.py writes
// oracle/_ref/ref_<version>.fatbin) and loaded through the CUDA driver API.  This file
// restates only the reference's host wrappers — launch shape (computeGridSize(n, 256):
// min(256, n) threads, ceil(n / threads) blocks), the cellStart memset, kernel order, the
// fill_cell launch of opt_src_v4/lib/mesh.cu:253-254 — and calls thrust::sort_by_key for
// sortParticles exactly as src/lib/mesh.cu:73-86 does.  Kernels are found by enumerating the
// module's functions and matching their mangled names.
//
// Used to generate the golden fixtures that pin the CPU oracle and to time the reference's
// CUDA solvers on the same GPU.  Never part of the product.
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include <cstdio>
#include <cstring>
#include <string>

namespace {

struct Ref {
    CUmodule mod = nullptr;
    CUfunction calc_hash = nullptr, reorder = nullptr, recover = nullptr, k1 = nullptr,
               k2 = nullptr, pred = nullptr, corr = nullptr, fill_cell = nullptr;
    CUdeviceptr par = 0;
    size_t par_bytes = 0;
    int num_cells = 0;
};

constexpr int kMaxModules = 8;
Ref g_mods[kMaxModules];
int g_count = 0;
char g_err[512];

int fail(const char* what, int code) {
    std::snprintf(g_err, sizeof(g_err), "%s (code %d)", what, code);
    return code ? code : -1;
}

Ref* get(int h) { return (h >= 0 && h < g_count) ? &g_mods[h] : nullptr; }

// Find the kernel whose mangled name is _Z<len><name>...
CUfunction find(CUfunction* all, unsigned count, const char* name) {
    std::string key = "_Z" + std::to_string(std::strlen(name)) + name;
    for (unsigned i = 0; i < count; i++) {
        const char* nm = nullptr;
        if (cuFuncGetName(&nm, all[i]) == CUDA_SUCCESS && nm &&
            std::strncmp(nm, key.c_str(), key.size()) == 0)
            return all[i];
    }
    return nullptr;
}

int launch_grid(CUfunction f, unsigned blocks, unsigned threads, void** args) {
    if (!blocks || !threads) return 0;
    CUresult r = cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, 0, nullptr, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : fail("cuLaunchKernel", (int)r);
}

// computeGridSize(n, 256, ...) of src/lib/mesh.cu:49-53
int launch(CUfunction f, int n, void** args) {
    if (n <= 0) return 0;
    unsigned t = (unsigned)(256 < n ? 256 : n);
    return launch_grid(f, (unsigned)((n + (int)t - 1) / (int)t), t, args);
}

}  // namespace

extern "C" const char* refh_error(void) { return g_err; }

// Load one fatbin; returns a handle >= 0 or a negative error.
extern "C" int refh_load(const char* fatbin_path) {
    if (g_count >= kMaxModules) return fail("too many modules", -6);
    cudaFree(0);  // make the runtime's primary context current
    Ref R;
    CUresult r = cuModuleLoad(&R.mod, fatbin_path);
    if (r != CUDA_SUCCESS) return -fail("cuModuleLoad", (int)r);
    unsigned count = 0;
    if ((r = cuModuleGetFunctionCount(&count, R.mod)) != CUDA_SUCCESS)
        return -fail("cuModuleGetFunctionCount", (int)r);
    CUfunction* all = new CUfunction[count];
    if ((r = cuModuleEnumerateFunctions(all, count, R.mod)) != CUDA_SUCCESS) {
        delete[] all;
        return -fail("cuModuleEnumerateFunctions", (int)r);
    }
    R.calc_hash = find(all, count, "calcHashD");
    R.reorder = find(all, count, "reorderD");
    R.recover = find(all, count, "recoverD");  // absent in v0..v4
    R.k1 = find(all, count, "computeBoundary_Delta_acoustic_D");
    R.k2 = find(all, count, "computeGovering_equationD");
    R.pred = find(all, count, "PC_predictionD");
    R.corr = find(all, count, "PC_correctionD");
    R.fill_cell = find(all, count, "fill_cell");  // v4 only
    delete[] all;
    if (!R.calc_hash || !R.reorder || !R.k1 || !R.k2 || !R.pred || !R.corr)
        return -fail("kernel not found in module", 2);
    if ((r = cuModuleGetGlobal(&R.par, &R.par_bytes, R.mod, "par")) != CUDA_SUCCESS)
        return -fail("cuModuleGetGlobal(par)", (int)r);
    g_mods[g_count] = R;
    return g_count++;
}

extern "C" int refh_has(int h, const char* what) {
    Ref* R = get(h);
    if (!R) return 0;
    if (!std::strcmp(what, "recover")) return R->recover != nullptr;
    if (!std::strcmp(what, "fill_cell")) return R->fill_cell != nullptr;
    return 0;
}

// The reference's cudaMemcpyToSymbol(par, temps, sizeof(SimParams)) (src/sph/sph_run.cu:105).
extern "C" int refh_set_params(int h, const void* simparams, size_t bytes, int num_cells) {
    Ref* R = get(h);
    if (!R) return fail("bad handle", -3);
    if (bytes != R->par_bytes) return fail("SimParams size mismatch", (int)R->par_bytes);
    CUresult r = cuMemcpyHtoD(R->par, simparams, bytes);
    R->num_cells = num_cells;
    return r == CUDA_SUCCESS ? 0 : fail("cuMemcpyHtoD(par)", (int)r);
}

extern "C" size_t refh_params_bytes(int h) {
    Ref* R = get(h);
    return R ? R->par_bytes : 0;
}

// calcHash (src/lib/mesh.cu:56-70)
extern "C" int refh_calc_hash(int h, float* pos, int* hash, int* index, int n) {
    void* args[] = {&pos, &hash, &index};
    return launch(get(h)->calc_hash, n, args);
}

// sortParticles (src/lib/mesh.cu:73-86)
extern "C" int refh_sort(int* hash, int* index, int n) {
    thrust::sort_by_key(thrust::device_ptr<int>(hash), thrust::device_ptr<int>(hash + n),
                        thrust::device_ptr<int>(index));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : fail("thrust::sort_by_key", (int)e);
}

// reorder (src/lib/mesh.cu:143-159; opt_src_v0/lib/mesh.cu:161-177 adds the permutation tables
// table_l / table_r; opt_src_v4/lib/mesh.cu:245-262 adds fill_cell and a device sync).
extern "C" int refh_reorder(int h, float* old_pos, float* old_vel, float* old_rho, float* old_p,
                            int* old_type, int* old_zone, float* s_pos, float* s_vel,
                            float* s_rho, float* s_p, int* s_type, int* s_zone, int* hash,
                            int* index, int* cell_start, int* cell_end, int n, int* table_l,
                            int* table_r) {
    Ref* R = get(h);
    if (cudaMemset(cell_start, 0xff, (size_t)R->num_cells * sizeof(int)) != cudaSuccess)
        return fail("cudaMemset", -5);
    int rc;
    if (table_l) {
        void* args[] = {&hash, &index, &cell_start, &cell_end, &old_pos, &old_vel, &old_rho,
                        &old_p, &old_type, &old_zone, &s_pos, &s_vel, &s_rho, &s_p, &s_type,
                        &s_zone, &table_l, &table_r};
        rc = launch(R->reorder, n, args);
    } else {
        void* args[] = {&hash, &index, &cell_start, &cell_end, &old_pos, &old_vel, &old_rho,
                        &old_p, &old_type, &old_zone, &s_pos, &s_vel, &s_rho, &s_p, &s_type,
                        &s_zone};
        rc = launch(R->reorder, n, args);
    }
    if (rc || !R->fill_cell) return rc;
    void* fargs[] = {&cell_start, &cell_end, &hash};
    rc = launch_grid(R->fill_cell, (unsigned)((R->num_cells + 256) / 256), 256, fargs);
    if (rc) return rc;
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail("cudaDeviceSynchronize", (int)e);
}

// recover (src/lib/mesh.cu:181-194)
extern "C" int refh_recover(int h, float* pos, float* vel, float* rho, float* p, int n,
                            int* index, int* type, int* zone, float* s_pos, float* s_vel,
                            float* s_rho, float* s_p, int* s_type, int* s_zone) {
    Ref* R = get(h);
    if (!R->recover) return fail("no recoverD in this module", -7);
    void* args[] = {&pos, &vel, &rho, &p, &index, &type, &zone, &s_pos, &s_vel, &s_rho, &s_p,
                    &s_type, &s_zone, &n};
    return launch(R->recover, n, args);
}

// SPH_NS_simpleversion (src/equation/ns.cu:5-28)
extern "C" int refh_ns(int h, float* s_pos, float* s_vel, float* s_rho, float* s_p, int* s_type,
                       float* rho_dt, float* vel_dt, int* cell_start, int* cell_end, int n,
                       int* hash, float* dofv, float* rhop_sum, float* w_sum) {
    Ref* R = get(h);
    void* a1[] = {&s_pos, &s_vel, &s_rho, &s_p, &s_type, &cell_start, &cell_end, &rhop_sum,
                  &w_sum, &n, &hash, &dofv};
    int rc = launch(R->k1, n, a1);
    if (rc) return rc;
    void* a2[] = {&s_pos, &s_vel, &s_p, &s_rho, &s_type, &rho_dt, &dofv, &vel_dt, &cell_start,
                  &cell_end, &n, &hash};
    return launch(R->k2, n, a2);
}

// PC_prediction / PC_correction (src/sph/sph_run.cu:521-550)
extern "C" int refh_pc_prediction(int h, float* s_pos, float* s_vel, float* s_rho, float* s_p,
                                  float* rho_dt, float* vel_dt, int* index, float* pos_tmp,
                                  float* vel_tmp, float* rho_tmp, int n, int* s_type) {
    void* args[] = {&s_pos, &s_vel, &s_rho, &s_p, &n, &rho_dt, &vel_dt, &pos_tmp, &vel_tmp,
                    &rho_tmp, &index, &s_type};
    return launch(get(h)->pred, n, args);
}

extern "C" int refh_pc_correction(int h, float* s_pos, float* s_vel, float* s_rho, float* s_p,
                                  float* rho_dt, float* vel_dt, int* index, float* pos_tmp,
                                  float* vel_tmp, float* rho_tmp, int n, int* s_type) {
    void* args[] = {&s_pos, &s_vel, &s_rho, &s_p, &rho_dt, &vel_dt, &pos_tmp, &vel_tmp,
                    &rho_tmp, &index, &n, &s_type};
    return launch(get(h)->corr, n, args);
}

extern "C" int refh_sync(void) {
    cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail(cudaGetErrorString(e), (int)e);
}
