// gi_drivers.cu -- the reference's three programs as headless library calls:
//   gi_generate_target_impactor  generateTargetImpactor.cu (body builder)
//   gi_impact_initialize         impactInitialization.cu (host only)
//   gi_impact_add_time           impactAddTime.cu (impact run / resume)
// They read and write the reference's files (gi_formats.cpp) and step with
// this library's fused force + kick-drift (gi_step), so a run directory
// made by either implementation can be continued by the other.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gi_internal.h"

namespace gi {

// pos += dp, vel += dv for every body (the recentering shift,
// impactAddTime.cu:443-452, float adds as the reference).
__global__ void __launch_bounds__(256)
shift_kernel(float4 *__restrict__ pos, float4 *__restrict__ vel, int n, float dpx, float dpy,
             float dpz, float dvx, float dvy, float dvz)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i], v = vel[i];
        p.x = __fadd_rn(p.x, dpx); p.y = __fadd_rn(p.y, dpy); p.z = __fadd_rn(p.z, dpz);
        v.x = __fadd_rn(v.x, dvx); v.y = __fadd_rn(v.y, dvy); v.z = __fadd_rn(v.z, dvz);
        pos[i] = p;
        vel[i] = v;
    }
}

}  // namespace gi

namespace {

int fail(int status, const std::string &msg) { return gi_internal_fail(status, msg.c_str()); }

int cuda_check(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return GI_OK;
    return fail(e == cudaErrorMemoryAllocation ? GI_ERR_OUT_OF_MEMORY : GI_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

std::string join(const char *dir, const char *name)
{
    std::string s = dir ? dir : ".";
    if (!s.empty() && s.back() != '/') s += '/';
    return s + name;
}

// A file-level call failed: keep its status, name the file.
int file_fail(int st, const std::string &path)
{
    if (st == GI_OK) return GI_OK;
    const char *what = st == GI_ERR_IO ? "cannot open or write" : "malformed or truncated";
    return fail(st, path + ": " + what);
}

// Device state of one driver run: context, state buffers, a force buffer.
struct DeviceRun {
    gi_ctx *ctx = nullptr;
    float *pos = nullptr, *vel = nullptr, *force = nullptr;
    unsigned char *scope = nullptr;
    int prev_device = -1, device = 0;
    ~DeviceRun()
    {
        cudaFree(pos);
        cudaFree(vel);
        cudaFree(force);
        cudaFree(scope);
        if (ctx) gi_ctx_destroy(ctx);
        if (prev_device >= 0 && prev_device != device) cudaSetDevice(prev_device);
    }
    int open(int dev, int n, bool with_force, bool with_scope)
    {
        device = dev;
        cudaGetDevice(&prev_device);
        if (int st = gi_ctx_create(&ctx, dev)) return st;
        if (cudaSetDevice(dev) != cudaSuccess) return fail(GI_ERR_NO_DEVICE, "cudaSetDevice failed");
        const size_t b = (size_t)(n > 0 ? n : 1) * 16;
        if (int st = cuda_check(cudaMalloc(&pos, b), "cudaMalloc pos")) return st;
        if (int st = cuda_check(cudaMalloc(&vel, b), "cudaMalloc vel")) return st;
        if (with_force)
            if (int st = cuda_check(cudaMalloc(&force, b), "cudaMalloc force")) return st;
        if (with_scope)
            if (int st = cuda_check(cudaMalloc(&scope, (size_t)(n > 0 ? n : 1)), "cudaMalloc scope"))
                return st;
        return GI_OK;
    }
    int upload(const std::vector<float> &p, const std::vector<float> &v)
    {
        if (int st = cuda_check(cudaMemcpy(pos, p.data(), p.size() * 4, cudaMemcpyHostToDevice),
                                "upload pos"))
            return st;
        return cuda_check(cudaMemcpy(vel, v.data(), v.size() * 4, cudaMemcpyHostToDevice),
                          "upload vel");
    }
    int download(std::vector<float> &p, std::vector<float> &v)
    {
        if (int st = cuda_check(cudaMemcpy(p.data(), pos, p.size() * 4, cudaMemcpyDeviceToHost),
                                "download pos"))
            return st;
        return cuda_check(cudaMemcpy(v.data(), vel, v.size() * 4, cudaMemcpyDeviceToHost),
                          "download vel");
    }
};

// Steps a run in pieces of at most 1024 so that a long phase is not one
// enormous call (the state stays on the device throughout).
int step_many(DeviceRun &d, const gi_run *runs, int nruns, const gi_pair_params *p, long long k)
{
    while (k > 0) {
        const int piece = (int)(k < 1024 ? k : 1024);
        if (int st = gi_step(d.ctx, d.pos, d.vel, runs, nruns, p, 1, piece, nullptr)) return st;
        k -= piece;
    }
    return GI_OK;
}

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" int gi_generate_target_impactor(int device, const char *setup_path, const char *info_dir,
                                           unsigned long long seed, gi_generate_report *report)
{
    if (!setup_path || !info_dir) return fail(GI_ERR_INVALID_ARG, "NULL path");
    gi_setup_generating setup;
    if (int st = gi_read_setup_generating(setup_path, &setup)) return file_fail(st, setup_path);
    gi_generation_plan plan;
    if (int st = gi_derive_units(&setup, &plan))
        return fail(st, "setup: body fractions must add to 1, n and the masses must be positive");
    if (!(setup.dt > 0.0)) return fail(GI_ERR_PARAMS, "setup: Dt must be positive");
    const gi_body_params &b = plan.body;
    const int n = b.n;
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n);
    long long redraws = 0;
    if (int st = gi_raw_bodies(seed, &b, pos.data(), vel.data(), &redraws))
        return fail(st, "raw bodies could not be placed");
    gi_force_separate_consts fc;
    gi_move_separate_consts mc;
    gi_separate_consts_from_body_params(&b, setup.dt, &fc, &mc);
    gi_pair_params p;
    gi_params_from_separate_consts(&fc, &p);
    // one run per body: the separate force has no cross-body pairs
    gi_run runs[2];
    const int n1 = b.nfe1 + b.nsi1;
    runs[0] = gi_run{0, n1, b.nfe1, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, setup.damp1};
    runs[1] = gi_run{n1, n - n1, b.nfe2, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, setup.damp2};
    gi_run rest[2] = {runs[0], runs[1]};
    rest[0].damp = rest[1].damp = 0.0f;
    const int nr = (n - n1) > 0 ? 2 : 1;

    // Phase of each step as the reference decides it: RunTime += Dt first,
    // then damped while RunTime < DampTime, damped rest while below
    // DampTime + DampRestTime, then spin rest (the spin is applied once, at
    // the first spin-rest step, between its force and its move); the run
    // ends after the step at which DampTime + DampRestTime + SpinRestTime <
    // RunTime (generateTargetImpactor.cu:666-749).
    long long count[3] = {0, 0, 0};
    {
        const double t_end = plan.damp_time + plan.damp_rest_time + plan.spin_rest_time;
        const long long limit = 2000000000LL;
        double t = 0.0;
        for (long long k = 0; k < limit; ++k) {
            t += setup.dt;
            const int ph = t < plan.damp_time ? 0 : (t < plan.damp_time + plan.damp_rest_time ? 1 : 2);
            ++count[ph];
            if (t_end < t) break;
        }
    }
    DeviceRun d;
    if (int st = d.open(device, n, true, false)) return st;
    if (int st = d.upload(pos, vel)) return st;
    const auto t0 = std::chrono::steady_clock::now();
    if (int st = step_many(d, runs, nr, &p, count[0])) return st;
    if (int st = step_many(d, rest, nr, &p, count[1])) return st;
    if (count[2] > 0) {
        if (int st = gi_forces(d.ctx, d.pos, d.vel, d.force, rest, nr, &p, 1, nullptr)) return st;
        if (int st = d.download(pos, vel)) return st;
        const float *axes[2] = {setup.spin1, setup.spin2};
        const float w[2] = {plan.spin1_w, plan.spin2_w};
        for (int body = 1; body <= 2; ++body)
            if (int st = gi_spin_body(pos.data(), vel.data(), &plan, body, axes[body - 1], w[body - 1]))
                return fail(st, "spin: the spin axis of a body is zero");
        if (int st = d.upload(pos, vel)) return st;
        if (int st = gi_move(d.ctx, d.pos, d.vel, d.force, rest, nr, nullptr)) return st;
        if (int st = step_many(d, rest, nr, &p, count[2] - 1)) return st;
    }
    if (int st = cuda_check(cudaDeviceSynchronize(), "step loop")) return st;
    const double secs = seconds_since(t0);
    if (int st = d.download(pos, vel)) return st;
    gi_zero_drift(pos.data(), vel.data(), &plan);
    std::string path = join(info_dir, "targetImpactorStats");
    if (int st = gi_write_target_impactor_stats(path.c_str(), &plan, &setup, setup.dt, pos.data(),
                                                vel.data()))
        return file_fail(st, path);
    path = join(info_dir, "targetImpactorParameters");
    if (int st = gi_write_body_params(path.c_str(), &b)) return file_fail(st, path);
    path = join(info_dir, "targetImpactorInitialPosVel");
    if (int st = gi_write_body_file(path.c_str(), pos.data(), vel.data(), n)) return file_fail(st, path);
    if (report) {
        report->damped_steps = count[0];
        report->rest_steps = count[1];
        report->spin_steps = count[2];
        report->steps = count[0] + count[1] + count[2];
        report->redraws = redraws;
        report->seconds = secs;
    }
    return GI_OK;
}

extern "C" int gi_impact_initialize(const char *info_dir, const char *setup_path,
                                    const char *impact_info_dir)
{
    if (!info_dir || !setup_path || !impact_info_dir) return fail(GI_ERR_INVALID_ARG, "NULL path");
    gi_body_params b;
    std::string path = join(info_dir, "targetImpactorParameters");
    if (int st = gi_read_body_params(path.c_str(), &b)) return file_fail(st, path);
    if (b.n < 0 || b.nfe1 < 0 || b.nsi1 < 0 || b.nfe2 < 0 || b.nsi2 < 0 ||
        (long long)b.nfe1 + b.nsi1 + b.nfe2 + b.nsi2 != b.n)
        return fail(GI_ERR_FORMAT, path + ": element counts do not add up");
    gi_setup_impact_init s;
    if (int st = gi_read_setup_impact_init(setup_path, &s)) return file_fail(st, setup_path);
    path = join(info_dir, "targetImpactorInitialPosVel");
    int nfile = 0;
    if (int st = gi_read_body_file(path.c_str(), nullptr, nullptr, 0, &nfile)) return file_fail(st, path);
    if (nfile < b.n) return fail(GI_ERR_FORMAT, path + ": fewer bodies than the parameters name");
    std::vector<float> p0(4 * (size_t)nfile), v0(4 * (size_t)nfile);
    if (int st = gi_read_body_file(path.c_str(), p0.data(), v0.data(), nfile, &nfile))
        return file_fail(st, path);
    std::vector<float> pos(4 * (size_t)b.n), vel(4 * (size_t)b.n);
    if (int st = gi_impact_initial_conditions(&b, &s, p0.data(), v0.data(), pos.data(), vel.data()))
        return fail(st, "impact initial conditions: bad parameters");
    path = join(impact_info_dir, "impactPosVel");
    std::remove(path.c_str());
    if (int st = gi_frames_append(path.c_str(), 0.0f, pos.data(), vel.data(), b.n))
        return file_fail(st, path);
    double stats[10];
    gi_system_stats_host(pos.data(), vel.data(), b.n, b.nfe1 + b.nfe2, b.mass_fe, b.mass_si, stats);
    path = join(impact_info_dir, "initialStatsFile");
    if (int st = gi_write_initial_stats(path.c_str(), &b, stats)) return file_fail(st, path);
    const float view[6] = {(float)stats[1], (float)stats[2], (float)stats[3],
                           (float)stats[4], (float)stats[5], (float)stats[6]};
    path = join(impact_info_dir, "viewCenteringInfo");
    if (int st = gi_write_view_centering(path.c_str(), view)) return file_fail(st, path);
    // keep a copy of the setup beside the results, as the reference does
    std::string text;
    if (FILE *in = std::fopen(setup_path, "rb")) {
        char buf[4096];
        size_t k;
        while ((k = std::fread(buf, 1, sizeof buf, in)) > 0) text.append(buf, k);
        std::fclose(in);
    }
    path = join(impact_info_dir, "setupImpactInitialization");
    if (FILE *out = std::fopen(path.c_str(), "wb")) {
        std::fwrite(text.data(), 1, text.size(), out);
        std::fclose(out);
    }
    return GI_OK;
}

extern "C" int gi_impact_add_time(int device, const char *info_dir, const char *setup_path,
                                  const char *impact_dir, gi_add_time_report *report)
{
    if (!info_dir || !setup_path || !impact_dir) return fail(GI_ERR_INVALID_ARG, "NULL path");
    gi_body_params b;
    std::string path = join(info_dir, "targetImpactorParameters");
    if (int st = gi_read_body_params(path.c_str(), &b)) return file_fail(st, path);
    gi_setup_add_time s;
    if (int st = gi_read_setup_add_time(setup_path, &s)) return file_fail(st, setup_path);
    if (!(s.dt > 0.0)) return fail(GI_ERR_PARAMS, "setup: Dt must be positive");
    const std::string info = join(impact_dir, "ImpactInformation");
    float view[6];
    path = join(info.c_str(), "viewCenteringInfo");
    if (int st = gi_read_view_centering(path.c_str(), view)) return file_fail(st, path);
    gi_force_collision_consts fc;
    gi_move_collision_consts mc;
    if (int st = gi_collision_consts_from_body_params(&b, s.dt, &fc, &mc))
        return fail(st, "targetImpactorParameters: element counts do not add up");
    gi_pair_params p;
    if (int st = gi_params_from_collision_consts(&fc, &p)) return st;
    const int n = b.n, nfe = fc.NFe;
    const std::string frames = join(info.c_str(), "impactPosVel");
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n);
    float t_file = 0.0f;
    if (int st = gi_frames_read(frames.c_str(), n, -1, &t_file, pos.data(), vel.data()))
        return file_fail(st, frames);
    // AdditionalTime: days -> seconds -> code units (impactAddTime.cu:120-124)
    const double additional = s.additional_time_days * 24.0 * 60.0 * 60.0 / b.unit_time;
    double run_time = (double)t_file;
    const double total_time = run_time + additional;
    if (!std::isfinite(total_time) || !(s.dt > 0.0))
        return fail(GI_ERR_PARAMS, "setup: AdditionalTime and Dt must be finite, Dt positive");
    const gi_run run{0, n, nfe, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, 0.0f};

    DeviceRun d;
    if (int st = d.open(device, n, false, true)) return st;
    if (int st = d.upload(pos, vel)) return st;
    const auto t0 = std::chrono::steady_clock::now();
    long long steps = 0, frames_written = 0, recenters = 0, pending = 0;
    int record_count = 0, recenter_count = 0;
    // The reference's loop (impactAddTime.cu:396-481): step, RunTime += Dt,
    // append a frame every RecordRate steps, recenter every RecenterRate
    // steps, stop after the step at which TotalRunTime < RunTime.  Steps
    // between two events run as one gi_step call.
    for (;;) {
        if (steps >= 2000000000LL) return fail(GI_ERR_PARAMS, "add time: more than 2e9 steps");
        ++steps;
        ++pending;
        run_time += s.dt;
        ++record_count;
        ++recenter_count;
        const bool record = record_count == s.record_rate;
        const bool recenter = recenter_count == s.recenter_rate;
        const bool done = total_time < run_time;
        if (record || recenter || done) {
            if (int st = step_many(d, &run, 1, &p, pending)) return st;
            pending = 0;
        }
        if (record) {
            if (int st = d.download(pos, vel)) return st;
            if (int st = gi_frames_append(frames.c_str(), (float)run_time, pos.data(), vel.data(), n))
                return file_fail(st, frames);
            ++frames_written;
            record_count = 0;
        }
        if (recenter) {
            double st0[15];
            if (int st = gi_diag_fp64(d.ctx, d.pos, d.vel, nullptr, 0, &run, &p, st0, nullptr))
                return st;
            const float dpx = view[0] - (float)st0[1], dpy = view[1] - (float)st0[2],
                        dpz = view[2] - (float)st0[3];
            const float dvx = view[3] - (float)st0[4], dvy = view[4] - (float)st0[5],
                        dvz = view[5] - (float)st0[6];
            gi::shift_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256>>>(
                reinterpret_cast<float4 *>(d.pos), reinterpret_cast<float4 *>(d.vel), n, dpx, dpy,
                dpz, dvx, dvy, dvz);
            if (int st = cuda_check(cudaGetLastError(), "recenter")) return st;
            ++recenters;
            recenter_count = 0;
        }
        if (done) break;
    }
    if (int st = cuda_check(cudaDeviceSynchronize(), "step loop")) return st;
    const double secs = seconds_since(t0);
    // final statistics (recordFinalImpactStat, impactBasicFunctions.h:883-1072)
    gi_earth_moon em;
    const int bounds[3] = {b.nfe1, b.nfe1 + b.nfe2, b.nfe1 + b.nfe2 + b.nsi1};
    const float touch = (float)(b.diameter * 1.5);
    if (int st = gi_find_earth_moon(d.ctx, d.pos, n, touch, bounds, nullptr, d.scope, &em, nullptr))
        return st;
    double S[4][15];
    for (int scope = 0; scope < 4; ++scope)
        if (int st = gi_diag_fp64(d.ctx, d.pos, d.vel, d.scope, scope, &run, &p, S[scope], nullptr))
            return st;
    path = join(impact_dir, "runStatsFile");
    if (int st = gi_write_run_stats(path.c_str(), &b, run_time, &em, S)) return file_fail(st, path);
    // the disk (not in the reference's statistics file; reported to the caller)
    gi_disk_info disk;
    double disk_stats[15];
    if (int st = gi_find_disk(d.ctx, d.pos, d.vel, &run, &p, d.scope, &disk, nullptr)) return st;
    if (int st = gi_diag_fp64(d.ctx, d.pos, d.vel, d.scope, 4, &run, &p, disk_stats, nullptr))
        return st;
    path = join(info.c_str(), "viewCenteringInfo");
    if (int st = gi_write_view_centering(path.c_str(), view)) return file_fail(st, path);
    if (report) {
        report->steps = steps;
        report->frames_written = frames_written;
        report->recenters = recenters;
        report->start_time = (double)t_file;
        report->end_time = run_time;
        report->seconds = secs;
        report->earth_moon = em;
        report->disk = disk;
        std::memcpy(report->disk_stats, disk_stats, sizeof disk_stats);
    }
    return GI_OK;
}
