// Native autotuner of the step's knobs (astro_autotune) and the batched
// step entry (astro_step_batched).
//
// The tuner times graph-replayed steps with dt = 0 (the particles never
// move, so every trial sees the same input) on the context's own particles
// and measures each setting's median relative acceleration error against
// the FP64 direct sum on sampled particles. Search: coordinate descent over
// the speed knobs (lbits, bucket, group_size, block_warps, sort_variant,
// walk_frontier),
// keeping the fastest setting whose error stays within
// max(target, 1.02 x the starting error); then every (open_delta_weight,
// far_ratio) pair, far_ratio rising until the error leaves
// max(0.8 x target, 1.02 x the starting error); then lbits, bucket,
// group_size, block_warps and walk_frontier once more within that bound. sort_variant is
// judged by the sort stage's own time. theta, the softening, the walk flags
// and the form are physics and stay as set; astro_autotune_keep also holds
// the knobs its caller names (a workload quoted at a given tree depth).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

namespace {

struct Knobs {
    uint32_t lbits, bucket, group_size, block_warps, sort_variant, walk_frontier;
    float far_ratio, open_delta_weight;
    bool operator==(const Knobs& o) const {
        return lbits == o.lbits && bucket == o.bucket && group_size == o.group_size &&
               block_warps == o.block_warps && sort_variant == o.sort_variant &&
               walk_frontier == o.walk_frontier && far_ratio == o.far_ratio &&
               open_delta_weight == o.open_delta_weight;
    }
};

struct Trial {
    Knobs k;
    double ms = 0, sort_ms = 0, err = 0;
};

enum Knob { kLbits, kBucket, kGroupSize, kBlockWarps, kSortVariant, kWalkFrontier };

class Tuner {
public:
    Tuner(astro_ctx* ctx, float target, uint32_t n_samples, uint32_t keep)
        : ctx_(ctx), target_(target), n_samples_(n_samples), keep_(keep) {}
    ~Tuner() {
        for (cudaEvent_t& e : ev_)
            if (e) cudaEventDestroy(e);
    }
    Tuner(const Tuner&) = delete;
    Tuner& operator=(const Tuner&) = delete;

    int run(const char* path);
    // The context's parameters before tuning, with its particles uploaded
    // again if a trial changed the tree depth.
    int restore(const astro_params& before);

private:
    astro_ctx* ctx_;
    float target_;
    uint32_t n_samples_;
    uint32_t keep_;  // ASTRO_TUNE_KEEP_* knobs held at the starting values
    astro_params base_{};
    std::vector<PositionMass> pm_;
    std::vector<VelocityRadius> vr_;
    std::vector<uint32_t> sizes_, samples_;
    std::vector<double> direct_;
    uint32_t steps_ = 3;
    std::vector<Trial> trials_;
    cudaEvent_t ev_[2] = {nullptr, nullptr};

    Knobs knobs_of(const astro_params& p) const {
        return {p.lbits, p.bucket, p.group_size ? p.group_size : 32u, p.block_warps ? p.block_warps : 4u,
                p.sort_variant, p.walk_frontier, p.far_ratio, p.open_delta_weight};
    }
    astro_params params_of(const Knobs& k) const {
        astro_params p = base_;
        p.lbits = k.lbits;
        p.bucket = k.bucket;
        p.group_size = k.group_size;
        p.block_warps = k.block_warps;
        p.sort_variant = k.sort_variant;
        p.walk_frontier = k.walk_frontier;
        p.far_ratio = k.far_ratio;
        p.open_delta_weight = k.open_delta_weight;
        return p;
    }
    int apply(const Knobs& k);
    int measure(const Knobs& k, Trial* t);
    std::vector<uint32_t> candidates(Knob knob) const;
    int sweep(Knob knob, double limit, Trial* best);
    int write(const char* path, const Trial& best, double bound, double acc_bound) const;
};

int Tuner::restore(const astro_params& before) {
    int r = astro_set_params(ctx_, &before);
    if (r != ASTRO_OK || ctx_->uploaded || pm_.empty()) return r;
    return sizes_.size() > 1
               ? astro_upload_systems(ctx_, pm_.data(), vr_.data(), sizes_.data(), (uint32_t)sizes_.size())
               : astro_upload(ctx_, pm_.data(), vr_.data(), nullptr, (uint32_t)pm_.size(),
                              (uint32_t)pm_.size());
}

// Applies a setting; a new tree depth needs the particles uploaded again.
int Tuner::apply(const Knobs& k) {
    const astro_params p = params_of(k);
    int r = astro_set_params(ctx_, &p);
    if (r != ASTRO_OK) return r;
    if (!ctx_->uploaded) {
        r = sizes_.size() > 1
                ? astro_upload_systems(ctx_, pm_.data(), vr_.data(), sizes_.data(), (uint32_t)sizes_.size())
                : astro_upload(ctx_, pm_.data(), vr_.data(), nullptr, (uint32_t)pm_.size(),
                               (uint32_t)pm_.size());
    }
    return r;
}

int Tuner::measure(const Knobs& k, Trial* t) {
    int r = apply(k);
    if (r != ASTRO_OK) return r;
    cudaStream_t st = ctx_->stream;
    // Warm-up, checked: a walk that needs larger buffers gets them here,
    // not inside the timed steps.
    if ((r = astro_step(ctx_, 0.0f, 3)) != ASTRO_OK) return r;
    if ((r = astro_synchronize(ctx_)) != ASTRO_OK) return r;
    cudaEventRecord(ev_[0], st);
    if ((r = astro_step(ctx_, 0.0f, steps_)) != ASTRO_OK) return r;
    cudaEventRecord(ev_[1], st);
    if ((r = astro_synchronize(ctx_)) != ASTRO_OK) return r;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
    t->k = k;
    t->ms = ms / steps_;
    // The sort stage alone: median of three stage sequences.
    float sort_ms[3];
    for (int i = 0; i < 3; ++i) {
        if ((r = astro_encode(ctx_)) != ASTRO_OK) return r;
        cudaEventRecord(ev_[0], st);
        if ((r = astro_sort(ctx_)) != ASTRO_OK) return r;
        cudaEventRecord(ev_[1], st);
        if ((r = astro_build(ctx_)) != ASTRO_OK || (r = astro_traverse(ctx_)) != ASTRO_OK ||
            (r = astro_integrate(ctx_, 0.0f)) != ASTRO_OK || (r = astro_synchronize(ctx_)) != ASTRO_OK)
            return r;
        cudaEventElapsedTime(&sort_ms[i], ev_[0], ev_[1]);
    }
    std::sort(sort_ms, sort_ms + 3);
    t->sort_ms = sort_ms[1];
    // Median relative error of the sampled accelerations.
    const uint32_t n = (uint32_t)pm_.size();
    std::vector<float> acc(4ull * n);
    if ((r = astro_encode(ctx_)) != ASTRO_OK || (r = astro_sort(ctx_)) != ASTRO_OK ||
        (r = astro_build(ctx_)) != ASTRO_OK || (r = astro_traverse(ctx_)) != ASTRO_OK ||
        (r = astro_read_accel(ctx_, acc.data(), n)) != ASTRO_OK ||
        (r = astro_integrate(ctx_, 0.0f)) != ASTRO_OK || (r = astro_synchronize(ctx_)) != ASTRO_OK)
        return r;
    std::vector<double> rel(samples_.size());
    for (size_t s = 0; s < samples_.size(); ++s) {
        const float* a = &acc[4ull * samples_[s]];
        const double* d = &direct_[3 * s];
        double e2 = 0, d2 = 0;
        for (int c = 0; c < 3; ++c) {
            e2 += ((double)a[c] - d[c]) * ((double)a[c] - d[c]);
            d2 += d[c] * d[c];
        }
        rel[s] = d2 > 0 ? std::sqrt(e2 / d2) : 0.0;
    }
    std::nth_element(rel.begin(), rel.begin() + rel.size() / 2, rel.end());
    t->err = rel[rel.size() / 2];
    trials_.push_back(*t);
    return ASTRO_OK;
}

std::vector<uint32_t> Tuner::candidates(Knob knob) const {
    switch (knob) {
        case kLbits: {
            // From about 8 particles per finest cell down to single occupancy,
            // within the 64-bit key beside the system bits.
            uint32_t nmax = 8;
            for (uint32_t s : sizes_) nmax = std::max(nmax, s);
            const uint32_t lo =
                std::max(3u, (uint32_t)std::ceil(std::log2((double)nmax / 8.0) / 3.0));
            uint32_t sysbits = 0;
            while ((1ull << sysbits) < sizes_.size()) ++sysbits;
            std::vector<uint32_t> c;
            for (uint32_t v : {lo, lo + 1, lo + 2, lo + 4, lo + 6}) {
                v = std::min(21u, v);
                if (3 * v + sysbits <= 64 && std::find(c.begin(), c.end(), v) == c.end()) c.push_back(v);
            }
            return c;
        }
        case kBucket: return {8, 16, 32, 64};
        case kGroupSize: return {8, 12, 16, 24, 32, 48, 64};
        case kBlockWarps: return {4, 8};
        case kSortVariant: {
            std::vector<uint32_t> v;
            for (uint32_t i = 1; i <= astro::sort_variant_count(); ++i) v.push_back(i);
            return v;
        }
        case kWalkFrontier: return {0, 1};
    }
    return {};
}

int Tuner::sweep(Knob knob, double limit, Trial* best) {
    if ((knob == kLbits && (keep_ & ASTRO_TUNE_KEEP_LBITS)) ||
        (knob == kGroupSize && (keep_ & ASTRO_TUNE_KEEP_GROUP_SIZE)))
        return ASTRO_OK;
    for (uint32_t v : candidates(knob)) {
        Knobs k = best->k;
        uint32_t* field = knob == kLbits ? &k.lbits : knob == kBucket ? &k.bucket
                          : knob == kGroupSize ? &k.group_size : knob == kBlockWarps ? &k.block_warps
                          : knob == kWalkFrontier ? &k.walk_frontier : &k.sort_variant;
        if (*field == v) continue;
        *field = v;
        Trial t;
        int r = measure(k, &t);
        if (r != ASTRO_OK) return r;
        const bool faster = knob == kSortVariant ? t.sort_ms < best->sort_ms : t.ms < best->ms;
        if (faster && t.err <= limit) *best = t;
    }
    return ASTRO_OK;
}

void put_knobs(std::string& s, const Knobs& k) {
    char b[256];
    std::snprintf(b, sizeof(b),
                  "{\"lbits\": %u, \"bucket\": %u, \"group_size\": %u, \"block_warps\": %u, "
                  "\"sort_variant\": %u, \"walk_frontier\": %u, \"far_ratio\": %.9g, "
                  "\"open_delta_weight\": %.9g}",
                  k.lbits, k.bucket, k.group_size, k.block_warps, k.sort_variant, k.walk_frontier,
                  (double)k.far_ratio, (double)k.open_delta_weight);
    s += b;
}

int Tuner::write(const char* path, const Trial& best, double bound, double acc_bound) const {
    std::string s = "{\"knobs\": ";
    put_knobs(s, best.k);
    char b[512];
    std::snprintf(b, sizeof(b),
                  ", \"ms\": %.9g, \"sort_ms\": %.9g, \"median_error\": %.9g, \"error_bound\": %.9g, "
                  "\"accuracy_knob_bound\": %.9g, \"steps_timed\": %u, \"n\": %zu, \"samples\": %zu, "
                  "\"trials\": [",
                  best.ms, best.sort_ms, best.err, bound, acc_bound, steps_, pm_.size(), samples_.size());
    s += b;
    for (size_t i = 0; i < trials_.size(); ++i) {
        s += i ? ", {\"knobs\": " : "{\"knobs\": ";
        put_knobs(s, trials_[i].k);
        std::snprintf(b, sizeof(b), ", \"ms\": %.9g, \"sort_ms\": %.9g, \"median_error\": %.9g}",
                      trials_[i].ms, trials_[i].sort_ms, trials_[i].err);
        s += b;
    }
    s += "]}\n";
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        ctx_->last_error = "autotune: cannot open the result file";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
    if (std::fclose(f) != 0 || !ok) {
        ctx_->last_error = "autotune: writing the result file failed";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    return ASTRO_OK;
}

int Tuner::run(const char* path) {
    base_ = ctx_->p;
    const uint32_t n = ctx_->n;
    sizes_ = ctx_->sys_sizes;
    pm_.resize(n);
    vr_.resize(n);
    int r = astro_download(ctx_, pm_.data(), vr_.data(), n);
    if (r != ASTRO_OK) return r;
    // Evenly spaced samples of the particles (upload order).
    const uint32_t ns = std::min(n, n_samples_);
    samples_.resize(ns);
    for (uint32_t s = 0; s < ns; ++s) samples_[s] = (uint32_t)(((uint64_t)s * n + n / (2 * ns)) / ns);
    direct_.assign(3ull * ns, 0.0);
    if ((r = astro_direct_accel_f64(ctx_, samples_.data(), ns, direct_.data())) != ASTRO_OK) return r;
    if (cudaEventCreate(&ev_[0]) != cudaSuccess || cudaEventCreate(&ev_[1]) != cudaSuccess) {
        ctx_->last_error = "autotune: cudaEventCreate failed";
        return ASTRO_ERR_CUDA;
    }

    Trial best;
    const Knobs start = knobs_of(base_);
    steps_ = 3;
    if ((r = measure(start, &best)) != ASTRO_OK) return r;
    // About 60 ms of timed steps per trial.
    steps_ = (uint32_t)std::min(60.0, std::max(3.0, std::floor(60.0 / std::max(best.ms, 1e-3))));
    trials_.clear();
    if ((r = measure(start, &best)) != ASTRO_OK) return r;
    const double bound = std::max((double)target_, 1.02 * best.err);
    const double acc_bound = std::max(0.8 * target_, 1.02 * best.err);
    for (Knob k : {kLbits, kBucket, kGroupSize, kBlockWarps, kSortVariant, kWalkFrontier})
        if ((r = sweep(k, bound, &best)) != ASTRO_OK) return r;
    // The accuracy knobs share one error budget.
    const Knobs base = best.k;
    for (float w : {1.0f, 0.85f, 0.7f, 0.5f}) {
        if (keep_ & ASTRO_TUNE_KEEP_ACCURACY) break;
        for (float f : {0.0f, 0.1f, 0.15f, 0.2f, 0.25f, 0.3f, 0.4f, 0.5f}) {
            Knobs k = base;
            k.open_delta_weight = w;
            k.far_ratio = f;
            if (k == best.k) continue;
            Trial t;
            if ((r = measure(k, &t)) != ASTRO_OK) return r;
            const bool ok = t.err <= acc_bound;
            if (ok && t.ms < best.ms) best = t;
            if (!ok) break;
        }
    }
    // The tree and launch knobs again (group boxes also decide far nodes).
    for (Knob k : {kLbits, kBucket, kGroupSize, kBlockWarps, kWalkFrontier})
        if ((r = sweep(k, acc_bound, &best)) != ASTRO_OK) return r;
    if ((r = apply(best.k)) != ASTRO_OK) return r;
    return path ? write(path, best, bound, acc_bound) : ASTRO_OK;
}

}  // namespace

extern "C" int astro_autotune_keep(astro_ctx* ctx, const char* path, float target, uint32_t samples,
                                   uint32_t keep) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (keep & ~(ASTRO_TUNE_KEEP_LBITS | ASTRO_TUNE_KEEP_GROUP_SIZE | ASTRO_TUNE_KEEP_ACCURACY)) {
        ctx->last_error = "autotune: unknown ASTRO_TUNE_KEEP_* bits";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    if (!ctx->uploaded) {
        ctx->last_error = "autotune: no particles uploaded";
        return ASTRO_ERR_STATE;
    }
    // Steps still unchecked finish (and rerun if their walk overflowed)
    // before the tuner reads the particles.
    if (int r = astro_synchronize(ctx); r != ASTRO_OK) return r;
    if (ctx->p.preset != ASTRO_PRESET_PHYSICAL) {
        ctx->last_error = "autotune: the REFERENCE preset's knobs are the reference's constants";
        return ASTRO_ERR_NOT_SUPPORTED;
    }
    if (!(target > 0.f) || !std::isfinite(target) || samples == 0) {
        ctx->last_error = "autotune: target must be > 0 and samples > 0";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    Tuner t(ctx, target, samples, keep);
    const astro_params before = ctx->p;
    const int r = t.run(path);
    if (r != ASTRO_OK) {
        const std::string why = ctx->last_error;
        t.restore(before);
        ctx->last_error = why;
    }
    return r;
}

extern "C" int astro_autotune_ex(astro_ctx* ctx, const char* path, float target, uint32_t samples) {
    return astro_autotune_keep(ctx, path, target, samples, 0u);
}

extern "C" int astro_autotune(astro_ctx* ctx, const char* path) {
    return astro_autotune_ex(ctx, path, 1e-3f, 1024);
}

extern "C" int astro_step_batched(astro_ctx* ctx, const uint32_t* sys_sizes, uint32_t nsys, float dt,
                                  uint32_t nsteps) {
    if (!ctx) return ASTRO_ERR_INVALID_ARGUMENT;
    if (!sys_sizes || nsys == 0) {
        ctx->last_error = "step_batched: null sizes or nsys == 0";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    if (!ctx->uploaded) {
        ctx->last_error = "step_batched: no particles uploaded";
        return ASTRO_ERR_STATE;
    }
    if (std::vector<uint32_t>(sys_sizes, sys_sizes + nsys) != ctx->sys_sizes) {
        ctx->last_error = "step_batched: sizes differ from the systems uploaded by astro_upload_systems";
        return ASTRO_ERR_INVALID_ARGUMENT;
    }
    return astro_step(ctx, dt, nsteps);
}
