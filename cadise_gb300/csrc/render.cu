// Render kernels: the FP32 megakernel, the wavefront stages, the FP64 film
// splat and the batched ray-query / camera kernels behind the C ABI.
//
// Replaces SamplingRenderer::render + EstimatorTileWork::work
// (source/core/renderer/sampling/samplingRenderer.cpp:33-68,
// source/core/renderer/render-work/estimatorTileWork.cpp:32-61): instead of
// tiles over host threads, a batch holds every path sample of one or more
// scenes for a range of sample indices; each path is independent and owns a
// counter-based random stream keyed by (seed, scene, pixel, sample).
//
// Wavefront schedule of one batch (replayed as one CUDA graph):
//   generate -> for b in [0, max_depth): { extend(b) || shadow(b) ; shade_k(b) for each BSDF kind }
//            -> extend(max_depth) || shadow(max_depth) -> splat
// Queues hold path ids; per-path state lives in SoA arrays indexed by path.
// Queue appends are warp-aggregated (ballot / match + one atomic per group).
#include "film.cuh"
#include "internal.h"
#include "pathtrace.cuh"
#include "radix.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

namespace cg {

template <bool COUNT, bool SPH>
__global__ void k_megakernel(RenderArgs a) {
    const BatchHeader h = *a.header;
    TraceCounters tc{0, 0}, ta{0, 0};
    uint32_t nc = 0, na = 0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < h.total_paths; p += gridDim.x * blockDim.x) {
        const PathId id = path_id(a.chunks, int(h.num_chunks), p);
        const SceneD& S = a.scenes[id.scene];
        Rng rng;
        float3 o, d;
        float2 fxy;
        primary_ray(S, id, h.seed, rng, &o, &d, &fxy);
        float3 L, Le, Ls;
        mk_path<COUNT, SPH>(S, o, d, rng, &L, &Le, &Ls, &tc, &ta, &nc, &na);
        a.wf.L[p] = make_float4(L.x, L.y, L.z, fxy.x);
        a.wf.Le[p] = make_float4(Le.x, Le.y, Le.z, 0.0f);
        a.wf.Ls[p] = make_float4(Ls.x, Ls.y, Ls.z, fxy.y);
    }
    count_flush<COUNT>(a.counters, tc, ta, nc, na);
}

// Per-path estimate for explicit film positions and keys (stream from draw 0).
__global__ void k_paths_explicit(const SceneD* scenes, int scene, const double* xy, const uint64_t* keys, uint32_t n,
                                 float* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const SceneD& S = scenes[scene];
        Rng rng;
        rng.key = keys[i];
        rng.ctr = 0;
        float3 o, d;
        camera_ray(S.cam, float(xy[2 * i]), float(xy[2 * i + 1]), &o, &d);
        float3 L, Le, Ls;
        TraceCounters tc{0, 0}, ta{0, 0};
        uint32_t nc = 0, na = 0;
        mk_path<false>(S, o, d, rng, &L, &Le, &Ls, &tc, &ta, &nc, &na);
        const float3 v = path_sample(L, Le, Ls);
        out[3 * i + 0] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    }
}

// ---------------------------------------------------------------- wavefront --
__global__ void k_wf_generate(RenderArgs a) {
    const BatchHeader h = *a.header;
    const WfBuffers& w = a.wf;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < h.total_paths; p += gridDim.x * blockDim.x) {
        const PathId id = path_id(a.chunks, int(h.num_chunks), p);
        const SceneD& S = a.scenes[id.scene];
        Rng rng;
        float3 o, d;
        float2 fxy;
        primary_ray(S, id, h.seed, rng, &o, &d, &fxy);
        w.ray_o[p] = make_float4(o.x, o.y, o.z, 0.0f);
        w.ray_d[p] = make_float4(d.x, d.y, d.z, 0.0f);
        w.thr[p] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(1));
        w.L[p] = make_float4(0.0f, 0.0f, 0.0f, fxy.x);
        w.Le[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.Ls[p] = make_float4(0.0f, 0.0f, 0.0f, fxy.y);
        w.meta[p] = make_uint4(uint32_t(id.scene), id.pixel, id.sample, rng.ctr);
        w.q_cont[0][p] = int(p);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) w.cnt[0] = int(h.total_paths);
}

// Append `p` to queue `key` (key < 0: no append); one atomic per group of
// lanes sharing a key.
CG_D void grouped_push(int* const* queues, int* counters, int key, int p) {
    const unsigned active = __activemask();
    const unsigned grp = __match_any_sync(active, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (lane == leader && key >= 0) base = atomicAdd(counters + key, __popc(grp));
    base = __shfl_sync(grp, base, leader);
    if (key >= 0) queues[key][base + __popc(grp & ((1u << lane) - 1u))] = p;
}

// After a closest-hit trace of queue entry p: a continuation hit is stored
// and its BSDF kind returned (the shade queue to join); an escaped
// continuation ray picks up the sky; a MIS ray that reaches its light adds
// the BSDF-sampling half of the NEE estimate.  Returns -1 when nothing is
// queued.
// ADJ (wavefront adjoint): the MIS half and its derivative by the light's
// radiance go to adj.mis_B / mis_X instead of L.
template <bool ADJ = false>
CG_D int extend_finish(const WfBuffers& w, const SceneD& S, int p, bool cont, float3 o, float3 d, bool hitp,
                       const HitD& hit, const AdjBufs* adj = nullptr) {
    if (cont) {
        if (hitp) {
            __stcs(&w.hit[p], make_float4(hit.t, __int_as_float(hit.slot), hit.u, hit.v));
            return shade_queue(S.materials[material_of_slot(S, hit.slot)].type);
        }
        if (S.env_light >= 0) {
            const float4 tw = w.thr[p];
            if (__float_as_int(tw.w) & 1) {
                const float3 e = f3(tw) * env_radiance(S, d);
                w.Le[p] = make_float4(e.x, e.y, e.z, 0.0f);
            }
        }
        return -1;
    }
    const float4 mb = w.mis_b[p];
    const int mlight = __float_as_int(mb.w);
    float3 add = splat3(0.0f), X = splat3(0.0f);
    bool has = false;
    int xlight = -1;
    if (hitp) {
        if (light_of_slot(S, hit.slot) == mlight) {
            const SurfaceD hs = surface_at(S, o, d, hit);
            const float4 ma = w.mis_a[p];
            add = mis_resolve(S, hs, o, f3(mb), f3(ma), ma.w, ADJ ? &X : nullptr);
            has = true;
            xlight = mlight;
        }
    } else if (mlight == S.env_light) {
        const float4 ma = w.mis_a[p];
        add = mis_resolve_env(S, d, f3(mb), f3(ma), ma.w);
        has = true;
    }
    if (ADJ) {
        if (has) {
            adj->mis_B[p] = make_float4(add.x, add.y, add.z, 1.0f);
            adj->mis_X[p] = make_float4(X.x, X.y, X.z, __int_as_float(xlight));
        }
        return -1;
    }
    if (has) {
        float4 L = w.L[p];
        L.x += add.x;
        L.y += add.y;
        L.z += add.z;
        w.L[p] = L;
    }
    return -1;
}

// MIS rays that meet their light (mis_light_hit): unless a primitive comes
// before the light's hit, the MIS term of extend_finish, added to L (ADJ:
// stored with its radiance derivative for the adjoint's gradient kernel).
template <bool COUNT, bool SPH, bool ADJ = false>
__global__ void k_wf_mis_occl(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    const int n = w.cnt[b * kCntStride + 11];
    const int* q = w.q_mocc[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nany = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = q[i];
        const SceneD& S = a.scenes[w.meta[p].x];
        const RayPre r = ray_prep(f3(w.ray_o[p]), f3(w.mis_d[p]), kRayEps, kFloatMax);
        const float4 mh = w.mis_h[p];
        const int slot = __float_as_int(mh.y);
        const int prim_l = slot >= 0 ? __float_as_int(ldg4(reinterpret_cast<const float4*>(S.tris + slot)).w) : 0x7FFFFFFF;
        if (COUNT) ++nany;
        if (occluded_before<COUNT, SPH>(S, r, mh.x, prim_l, slot, &tc)) continue;
        const float4 mb = w.mis_b[p], ma = w.mis_a[p];
        float3 add, X = splat3(0.0f);
        int xlight = -1;
        if (slot >= 0) {
            HitD hit;
            hit.t = mh.x;
            hit.slot = slot;
            hit.u = mh.z;
            hit.v = mh.w;
            const SurfaceD hs = surface_at(S, r.o, r.d, hit);
            add = mis_resolve(S, hs, r.o, f3(mb), f3(ma), ma.w, ADJ ? &X : nullptr);
            xlight = __float_as_int(mb.w);
        } else {
            add = mis_resolve_env(S, r.d, f3(mb), f3(ma), ma.w);
        }
        if (ADJ) {
            a.adj.mis_B[p] = make_float4(add.x, add.y, add.z, 1.0f);
            a.adj.mis_X[p] = make_float4(X.x, X.y, X.z, __int_as_float(xlight));
            continue;
        }
        float4 L = w.L[p];
        L.x += add.x;
        L.y += add.y;
        L.z += add.z;
        w.L[p] = L;
    }
    count_flush<COUNT>(a.counters, TraceCounters{0, 0}, tc, 0, nany);
}

// ADJ: marks an unoccluded shadow ray in sh_c.w for the adjoint's gradient kernel.
template <bool ADJ = false>
CG_D void shadow_finish(const WfBuffers& w, int p, bool occluded) {
    if (occluded) return;
    const float4 c = w.sh_c[p];
    if (ADJ) {
        w.sh_c[p] = make_float4(c.x, c.y, c.z, 1.0f);
        return;
    }
    float4 Ls = w.Ls[p];
    Ls.x += c.x;
    Ls.y += c.y;
    Ls.z += c.z;
    w.Ls[p] = Ls;
}

// Queue entry i of a closest-hit pass: its path and whether it is a
// continuation ray (else a MIS ray); SORTED reads the reordered queue.
template <bool SORTED>
CG_D int extend_entry(const RenderArgs& a, const int* qc, const int* qm, int ncont, int i, bool* cont) {
    if (SORTED) {
        const uint32_t e = a.sorted[i];
        *cont = (e >> 31) == 0u;
        return int(e & 0x7FFFFFFFu);
    }
    *cont = i < ncont;
    return *cont ? qc[i] : qm[i - ncont];
}

CG_D uint32_t spread9(uint32_t v) {
    uint32_t x = v & 0x1FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Sort keys of a closest-hit pass's queue (tuning.reorder): the direction's
// octant above the Morton code of the origin in the scene bounds (`bits` per
// axis, at most 9), so that sorted neighbours leave nearby points in similar
// directions.  Values: path | 0x80000000 for a MIS ray.  Writes the entry
// count for the sort.
__global__ void k_ray_keys(RenderArgs a, int b, int bits, uint32_t* keys, uint32_t* vals, uint32_t* n_out) {
    const WfBuffers& w = a.wf;
    const int* cnt = w.cnt + b * kCntStride;
    const int ncont = cnt[0], n = ncont + cnt[1];
    const int* qc = w.q_cont[b & 1];
    const int* qm = w.q_mis[b & 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_out = uint32_t(n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool cont = i < ncont;
        const int p = cont ? qc[i] : qm[i - ncont];
        const float3 o = f3(w.ray_o[p]);
        const float3 d = cont ? f3(w.ray_d[p]) : f3(w.mis_d[p]);
        const SceneD& S = a.scenes[w.meta[p].x];
        const float u[3] = {(o.x - S.bounds_lo.x) * S.bounds_inv.x, (o.y - S.bounds_lo.y) * S.bounds_inv.y,
                            (o.z - S.bounds_lo.z) * S.bounds_inv.z};
        const float cells = float((1 << bits) - 1);
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) q[k] = uint32_t(fminf(fmaxf(u[k], 0.0f), 1.0f) * cells);
        const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
        keys[i] = (oct << (3 * bits)) | (spread9(q[0]) << 2) | (spread9(q[1]) << 1) | spread9(q[2]);
        vals[i] = uint32_t(p) | (cont ? 0u : 0x80000000u);
    }
}

template <bool COUNT, bool SPH, bool ADJ = false, bool SORTED = false>
__global__ void k_wf_extend(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int ncont = cnt[0], nmis = cnt[1];
    const int n = ncont + nmis;
    const int* qc = w.q_cont[b & 1];
    const int* qm = w.q_mis[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nclosest = 0;
    int* const* qmat = w.q_mat;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool cont;
        const int p = extend_entry<SORTED>(a, qc, qm, ncont, i, &cont);
        const SceneD& S = a.scenes[w.meta[p].x];
        const float3 o = f3(w.ray_o[p]);
        const float3 d = cont ? f3(w.ray_d[p]) : f3(w.mis_d[p]);
        const RayPre r = ray_prep(o, d, kRayEps, kFloatMax);
        HitD hit;
        if (COUNT) ++nclosest;
        const bool hitp = traverse_warp<COUNT, SPH>(S, r, &hit, &tc);
        const int key = extend_finish<ADJ>(w, S, p, cont, o, d, hitp, hit, &a.adj);
        grouped_push(qmat, cnt + 3, key, p);
    }
    count_flush<COUNT>(a.counters, tc, TraceCounters{0, 0}, nclosest, 0);
}

template <bool COUNT, bool SPH, bool ADJ = false>
__global__ void k_wf_shadow(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    const int n = w.cnt[b * kCntStride + 2];
    const int* q = w.q_shadow[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nany = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = q[i];
        const SceneD& S = a.scenes[w.meta[p].x];
        const float4 sd = w.sh_d[p];
        const RayPre r = ray_prep(f3(w.ray_o[p]), f3(sd), kRayEps, sd.w);
        HitD hit;
        if (COUNT) ++nany;
        shadow_finish<ADJ>(w, p, traverse<true, COUNT, SPH>(S, r, &hit, &tc));
    }
    count_flush<COUNT>(a.counters, TraceCounters{0, 0}, tc, 0, nany);
}

// Persistent variants: each lane takes rays from the queue through a
// warp-aggregated counter and, whenever its ray finishes, the next one, so no
// lane idles while the warp's longest ray is still traversing.
constexpr int kStepsPerFetch = 4;

// Hands the lanes in `need` consecutive entries of [0, n); returns this lane's
// entry or -1 when the queue is drained.
CG_D int warp_take(int* work, bool need, int n) {
    const unsigned mask = __activemask();
    const unsigned nb = __ballot_sync(mask, need);
    if (nb == 0) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(nb) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(work, __popc(nb));
    base = __shfl_sync(mask, base, leader);
    if (!need) return -1;
    const int k = base + __popc(nb & ((1u << lane) - 1u));
    return k < n ? k : -1;
}

template <bool COUNT, bool SPH>
__global__ void k_wf_extend_dyn(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int ncont = cnt[0], nmis = cnt[1];
    const int n = ncont + nmis;
    const int* qc = w.q_cont[b & 1];
    const int* qm = w.q_mis[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nclosest = 0;
    int* const* qmat = w.q_mat;
    TravState st;
    RayPre r;
    int i = -1, p = -1;
    bool drained = false;
    float3 o = splat3(0.0f), d = splat3(0.0f);
    for (;;) {
        const bool need = i < 0 && !drained;
        const int k = warp_take(cnt + 8, need, n);
        if (need) {
            if (k < 0) {
                drained = true;
            } else {
                i = k;
                const bool cont = i < ncont;
                p = cont ? qc[i] : qm[i - ncont];
                o = f3(w.ray_o[p]);
                d = cont ? f3(w.ray_d[p]) : f3(w.mis_d[p]);
                r = ray_prep(o, d, kRayEps, kFloatMax);
                trav_begin(st, r, a.scenes[w.meta[p].x].visit_budget);
                if (COUNT) ++nclosest;
            }
        }
        if (__all_sync(__activemask(), i < 0)) break;
        if (i >= 0) {
            const SceneD& S = a.scenes[w.meta[p].x];
            for (int s = 0; s < kStepsPerFetch && !st.done; ++s) trav_step<false, COUNT, SPH>(S, r, st, &tc);
            if (st.done) {
                HitD hit;
                hit.slot = st.hslot;
                hit.t = st.tcur;
                hit.u = st.hu;
                hit.v = st.hv;
                const int key = extend_finish(w, S, p, i < ncont, o, d, st.hslot >= 0, hit);
                grouped_push(qmat, cnt + 3, key, p);
                i = -1;
            }
        }
    }
    count_flush<COUNT>(a.counters, tc, TraceCounters{0, 0}, nclosest, 0);
}

// Persistent closest-hit pass: the while-while traversal of traverse_warp
// with dynamic ray fetch (Aila & Laine 2009).  A lane keeps its ray across
// rounds; after each round of leaves, once fewer than a.refill_closest lanes
// of the warp still hold an unfinished ray (the autotuned compaction
// threshold), the finished lanes store their hits and take the next rays of
// the queue, so lanes do not idle until the warp's longest ray is done.
// Same hits as the other extend kernels (closer_hit).

// At most 56 registers a thread (a few spilled values, in the ray set-up):
// 18 blocks of 64 threads fit an SM instead of 12, and the closest-hit pass
// then runs beside the any-hit pass with more warps to hide its L1 / L2
// latency (samples/s on the 1 M-triangle frame: +4.5 % at 64 registers,
// +7.0 % at 56, against the uncapped 75).
template <bool COUNT, bool SPH, bool SORTED = false, bool ADJ = false>
__global__ void __maxnreg__(56) k_wf_extend_pww(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int ncont = cnt[0], nmis = cnt[1];
    const int n = ncont + nmis;
    const int* qc = w.q_cont[b & 1];
    const int* qm = w.q_mis[b & 1];
    int* const* qmat = w.q_mat;
    TraceCounters tc{0, 0};
    uint32_t nclosest = 0;
    SharedStack<true> stack;
    stack.bind();
    int sp = 0;
    RayPre r{};
    float tcur = 0.0f, hu = 0.0f, hv = 0.0f;
    int hslot = -1;
    uint32_t cur = kNoEntry, leaf = kNoEntry;
    int i = -1, p = -1;  // queue entry and path of this lane's ray (i < 0: none)
    bool cont = false;   // continuation ray (else MIS ray)
    bool drained = false;
    uint32_t left = 0;  // node and leaf visits this ray has left (over_budget)
    auto pop = [&]() -> uint32_t {
        while (sp > 0) {
            --sp;
            if (stack.dist(sp) <= tcur * 1.00000036f) return stack.entry(sp);
        }
        return kNoEntry;
    };
    for (;;) {
        const bool need = i < 0 && !drained;
        const int k = warp_take(cnt + 8, need, n);
        if (need) {
            if (k < 0) {
                drained = true;
            } else {
                i = k;
                p = extend_entry<SORTED>(a, qc, qm, ncont, i, &cont);
                const float3 o = f3(__ldcs(&w.ray_o[p]));
                const float3 d = cont ? f3(__ldcs(&w.ray_d[p])) : f3(__ldcs(&w.mis_d[p]));
                r = ray_prep(o, d, kRayEps, kFloatMax);
                tcur = r.tmax;
                hslot = -1;
                hu = hv = 0.0f;
                cur = 0;
                leaf = kNoEntry;
                sp = 0;
                left = a.scenes[__ldcs(&w.meta[p].x)].visit_budget;
                if (COUNT) ++nclosest;
            }
        }
        if (__all_sync(__activemask(), i < 0)) break;
        if (i < 0) continue;
        const SceneD& S = a.scenes[__ldcs(&w.meta[p].x)];
        for (;;) {
            while (cur != kNoEntry && !entry_is_leaf(cur)) {
                if (over_budget(S, left)) {
                    cur = leaf = kNoEntry;
                    break;
                }
                cur = visit_node<false, COUNT, false>(S, r, cur, tcur, stack, sp, &tc);
                if (cur == kNoEntry) cur = pop();
                if (leaf == kNoEntry && cur != kNoEntry && entry_is_leaf(cur)) {
                    leaf = cur;
                    cur = pop();
                }
                if (!__any_sync(__activemask(), leaf == kNoEntry)) break;
            }
            if (leaf == kNoEntry) {
                if (cur == kNoEntry) break;  // the ray is done
                leaf = cur;
                cur = pop();
            }
            while (leaf != kNoEntry) {
                if (over_budget(S, left)) {
                    cur = leaf = kNoEntry;
                    break;
                }
                visit_leaf<false, COUNT, SPH, true>(S, r, leaf, tcur, hslot, hu, hv, &tc);
                leaf = kNoEntry;
                if (cur != kNoEntry && entry_is_leaf(cur)) {
                    leaf = cur;
                    cur = pop();
                }
            }
            if (cur == kNoEntry) break;  // the ray is done
            if (__popc(__activemask()) < a.refill_closest) break;
        }
        if (cur == kNoEntry && leaf == kNoEntry) {
            if (hu != 0.0f) {
                // two primitives within the tie window: k_wf_ties decides
                w.q_tie[atomicAdd(cnt + 12, 1)] = cont ? p : int(uint32_t(p) | 0x80000000u);
            } else {
                HitD hit;
                hit.t = tcur;
                hit.slot = hslot;
                // the shading recomputes the surface coordinates from the hit
                // point (hit_point), so the traversal's need not be kept
                hit.u = 0.0f;
                hit.v = 0.0f;
                const int key = extend_finish<ADJ>(w, S, p, cont, r.o, r.d, hslot >= 0, hit, &a.adj);
                grouped_push(qmat, cnt + 3, key, p);
            }
            i = -1;
        }
    }
    count_flush<COUNT>(a.counters, tc, TraceCounters{0, 0}, nclosest, 0);
}

constexpr int kTieBlock = 64;

// Closest-hit rays the persistent pass left to this kernel (q_tie): two
// primitives within the tie window of each other, which tie_prefers orders
// by the reference's own test and tie order.  Traced again with the per-ray
// traversal (closer_hit / tie_prefers, wide culling), then finished as the
// persistent pass finishes its other rays.  It runs beside the any-hit pass
// (on the other stream), and its grid strides over however few rays it got.
template <bool COUNT, bool SPH, bool ADJ = false>
__global__ void k_wf_ties(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int n = cnt[12];
    int* const* qmat = w.q_mat;
    TraceCounters tc{0, 0};
    uint32_t nties = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (COUNT) ++nties;
        const int e = w.q_tie[i];
        const bool cont = e >= 0;
        const int p = e & 0x7FFFFFFF;
        const SceneD& S = a.scenes[w.meta[p].x];
        const float3 o = f3(w.ray_o[p]);
        const float3 d = cont ? f3(w.ray_d[p]) : f3(w.mis_d[p]);
        const RayPre r = ray_prep(o, d, kRayEps, kFloatMax);
        HitD hit;
        const bool hitp = traverse<false, COUNT, SPH>(S, r, &hit, &tc);
        hit.u = 0.0f;
        hit.v = 0.0f;
        const int key = extend_finish<ADJ>(w, S, p, cont, o, d, hitp, hit, &a.adj);
        grouped_push(qmat, cnt + 3, key, p);
    }
    count_flush<COUNT>(a.counters, tc, TraceCounters{0, 0}, 0, 0);
    if (COUNT && nties) atomicAdd(a.counters + 6, (unsigned long long)nties);
}

// Persistent any-hit pass: k_wf_extend_pww's while-while traversal with
// dynamic ray fetch for the shadow rays; a ray ends at its first hit.  The
// refill threshold is a.refill_any.

template <bool COUNT, bool SPH, bool ADJ = false>
__global__ void k_wf_shadow_pww(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int n = cnt[2];
    const int* q = w.q_shadow[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nany = 0;
    SharedStack<false> stack;
    stack.bind();
    int sp = 0;
    RayPre r{};
    float tcur = 0.0f, hu = 0.0f, hv = 0.0f;
    int hslot = -1;
    uint32_t cur = kNoEntry, leaf = kNoEntry;
    int i = -1, p = -1;
    bool occluded = false, drained = false;
    uint32_t left = 0;  // node and leaf visits this ray has left (over_budget)
    auto pop = [&]() -> uint32_t {
        if (sp > 0) return stack.entry(--sp);
        return kNoEntry;
    };
    for (;;) {
        const bool need = i < 0 && !drained;
        const int k = warp_take(cnt + 9, need, n);
        if (need) {
            if (k < 0) {
                drained = true;
            } else {
                i = k;
                p = q[i];
                const float4 sd = __ldcs(&w.sh_d[p]);
                r = ray_prep(f3(__ldcs(&w.ray_o[p])), f3(sd), kRayEps, sd.w);
                tcur = r.tmax;
                hslot = -1;
                cur = 0;
                leaf = kNoEntry;
                sp = 0;
                occluded = false;
                left = a.scenes[__ldcs(&w.meta[p].x)].visit_budget;
                if (COUNT) ++nany;
            }
        }
        if (__all_sync(__activemask(), i < 0)) break;
        if (i < 0) continue;
        const SceneD& S = a.scenes[__ldcs(&w.meta[p].x)];
        for (;;) {
            while (cur != kNoEntry && !entry_is_leaf(cur)) {
                if (over_budget(S, left)) {
                    cur = leaf = kNoEntry;
                    break;
                }
                cur = visit_node<true, COUNT>(S, r, cur, tcur, stack, sp, &tc);
                if (cur == kNoEntry) cur = pop();
                if (leaf == kNoEntry && cur != kNoEntry && entry_is_leaf(cur)) {
                    leaf = cur;
                    cur = pop();
                }
                if (!__any_sync(__activemask(), leaf == kNoEntry)) break;
            }
            if (leaf == kNoEntry) {
                if (cur == kNoEntry) break;  // the ray is done: unoccluded
                leaf = cur;
                cur = pop();
            }
            while (leaf != kNoEntry) {
                if (over_budget(S, left)) {
                    cur = leaf = kNoEntry;
                    break;
                }
                if (visit_leaf<true, COUNT, SPH>(S, r, leaf, tcur, hslot, hu, hv, &tc)) {
                    occluded = true;
                    cur = leaf = kNoEntry;
                    break;
                }
                leaf = kNoEntry;
                if (cur != kNoEntry && entry_is_leaf(cur)) {
                    leaf = cur;
                    cur = pop();
                }
            }
            if (cur == kNoEntry) break;  // the ray is done
            if (__popc(__activemask()) < a.refill_any) break;
        }
        if (cur == kNoEntry && leaf == kNoEntry) {
            shadow_finish<ADJ>(w, p, occluded);
            i = -1;
        }
    }
    count_flush<COUNT>(a.counters, TraceCounters{0, 0}, tc, 0, nany);
}

template <bool COUNT, bool SPH>
__global__ void k_wf_shadow_dyn(RenderArgs a, int b) {
    const WfBuffers& w = a.wf;
    int* cnt = w.cnt + b * kCntStride;
    const int n = cnt[2];
    const int* q = w.q_shadow[b & 1];
    TraceCounters tc{0, 0};
    uint32_t nany = 0;
    TravState st;
    RayPre r;
    int i = -1, p = -1;
    bool drained = false;
    for (;;) {
        const bool need = i < 0 && !drained;
        const int k = warp_take(cnt + 9, need, n);
        if (need) {
            if (k < 0) {
                drained = true;
            } else {
                i = k;
                p = q[i];
                const float4 sd = w.sh_d[p];
                r = ray_prep(f3(w.ray_o[p]), f3(sd), kRayEps, sd.w);
                trav_begin(st, r, a.scenes[w.meta[p].x].visit_budget);
                if (COUNT) ++nany;
            }
        }
        if (__all_sync(__activemask(), i < 0)) break;
        if (i >= 0) {
            const SceneD& S = a.scenes[w.meta[p].x];
            for (int s = 0; s < kStepsPerFetch && !st.done; ++s) trav_step<true, COUNT, SPH>(S, r, st, &tc);
            if (st.done) {
                shadow_finish(w, p, st.hslot >= 0);
                i = -1;
            }
        }
    }
    count_flush<COUNT>(a.counters, TraceCounters{0, 0}, tc, 0, nany);
}

// ------------------------------------------------------ wavefront adjoint --
// FP64 block sums of the few roughness / radiance gradients in shared memory
// ([0, nmat) roughness, then 3 per area light), flushed once per block.
CG_D void adj_shared_zero(double* sh, const AdjBufs& A) {
    for (int i = threadIdx.x; i < A.nmat + 3 * A.nlight; i += blockDim.x) sh[i] = 0.0;
    __syncthreads();
}
CG_D void adj_shared_flush(double* sh, const AdjBufs& A) {
    __syncthreads();
    for (int i = threadIdx.x; i < A.nmat; i += blockDim.x)
        if (sh[i] != 0.0) atomicAdd(A.g_rough + i, sh[i]);
    for (int i = threadIdx.x; i < 3 * A.nlight; i += blockDim.x)
        if (sh[A.nmat + i] != 0.0) atomicAdd(A.g_rad + i, sh[A.nmat + i]);
}
CG_D void adj_add(double* sh, int i, double v) {
    if (v != 0.0) atomicAdd(sh + i, v);
}
CG_D float3 adj_delta(const AdjBufs& A, uint32_t pixel) {
    return mk(A.dLdI[3 * pixel] * A.inv_spp, A.dLdI[3 * pixel + 1] * A.inv_spp, A.dLdI[3 * pixel + 2] * A.inv_spp);
}

// The adjoint's part of shading vertex b of path p (the replay of adjoint.cuh,
// split at the point where the vertex's shadow and MIS rays are traced): the
// emission term's radiance gradient now, the rest kept for k_adj_vertex.
// Returns whether the path carries gradient (finite total, nonzero weight).
CG_D bool adj_vertex_begin(const RenderArgs& a, double* sh, const SceneD& S, const SurfaceD& si, const VertexPlan& pl,
                           float4 tw, int p, uint32_t pixel) {
    const AdjBufs& A = a.adj;
    const float3 delta = adj_delta(A, pixel);
    if (!finite3(f3(A.Ltot[p])) || is_zero(delta)) return false;
    const bool ce = (__float_as_int(tw.w) & 1) != 0;
    if (si.light >= 0 && si.light < A.nlight && ce && can_emit(S.lights[si.light], si.wi, si.Ns)) {
        const float3 gx = delta * f3(tw);
        adj_add(sh + A.nmat, 3 * si.light + 0, gx.x);
        adj_add(sh + A.nmat, 3 * si.light + 1, gx.y);
        adj_add(sh + A.nmat, 3 * si.light + 2, gx.z);
    }
    const float4 acc = A.acc[p];
    A.acc[p] = make_float4(acc.x + pl.emit.x, acc.y + pl.emit.y, acc.z + pl.emit.z, 0.0f);
    const MaterialD& m = S.materials[si.material];
    uint32_t bits = uint32_t(si.material) | (pl.shadow ? kAdjShadow : 0u) | (pl.mis ? kAdjMis : 0u) |
                    (pl.cont ? kAdjCont : 0u);
    if (m.type == BSDF_LAMBERTIAN && m.albedo_tex >= 0) {
        const TextureD& tex = S.textures[m.albedo_tex];
        const float3 alb = texture_rgb(tex, si.uvw);
        A.st_a[p] = make_float4(alb.x, alb.y, alb.z, __int_as_float(3 * texel_index(tex, si.uvw)));
        bits |= kAdjTexel;
    }
    float gs = 0.0f, gb = 0.0f, gc = 0.0f;
    if (m.type == BSDF_CONDUCTOR || m.type == BSDF_DIELECTRIC_GGX) {
        if (pl.shadow) gs = dlogf_droughness(m, si.wi, pl.sdir, si.Ns);
        if (pl.mis) gb = dlogf_droughness(m, si.wi, pl.mdir, si.Ns);
        if (pl.cont) gc = dlogf_droughness(m, si.wi, pl.cdir, si.Ns);
        bits |= kAdjGgx;
    }
    A.st_b[p] = make_float4(gs, gb, gc, __uint_as_float(bits));
    if (pl.shadow) A.st_c[p] = make_float4(pl.sx.x, pl.sx.y, pl.sx.z, __int_as_float(pl.slight));
    if (pl.mis) A.mis_B[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return true;
}

// Vertices of bounce b, once their shadow (bounce b + 1 shadow pass) and MIS
// (bounce b + 1 extend pass) rays are traced: A, B and the radiance of the
// vertices after this one (R = Ltot - acc - A - B) give the texel, roughness
// and radiance terms of adjoint.cuh.
__global__ void k_adj_vertex(RenderArgs a, int b) {
    extern __shared__ double sh[];
    const WfBuffers& w = a.wf;
    const AdjBufs& A = a.adj;
    adj_shared_zero(sh, A);
    const int n = w.cnt[(b + 1) * kCntStride + 10];
    const int* q = A.q_vtx[b & 1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = q[i];
        const uint4 meta = w.meta[p];
        const SceneD& S = a.scenes[meta.x];
        const float3 delta = adj_delta(A, meta.y);
        const float4 sb = A.st_b[p];
        const uint32_t bits = __float_as_uint(sb.w);
        const int mat = int(bits & 0xFFFFu);
        float3 Av = splat3(0.0f), Bv = splat3(0.0f);
        if (bits & kAdjShadow) {
            const float4 c = w.sh_c[p];
            if (c.w != 0.0f) {
                Av = f3(c);
                const float4 sc = A.st_c[p];
                const int slight = __float_as_int(sc.w);
                if (slight < A.nlight) {
                    const float3 gx = delta * f3(sc);
                    adj_add(sh + A.nmat, 3 * slight + 0, gx.x);
                    adj_add(sh + A.nmat, 3 * slight + 1, gx.y);
                    adj_add(sh + A.nmat, 3 * slight + 2, gx.z);
                }
            }
        }
        if (bits & kAdjMis) {
            const float4 mb = A.mis_B[p];
            if (mb.w != 0.0f) {
                Bv = f3(mb);
                const float4 mx = A.mis_X[p];
                const int xl = __float_as_int(mx.w);
                if (xl >= 0 && xl < A.nlight) {
                    const float3 gx = delta * f3(mx);
                    adj_add(sh + A.nmat, 3 * xl + 0, gx.x);
                    adj_add(sh + A.nmat, 3 * xl + 1, gx.y);
                    adj_add(sh + A.nmat, 3 * xl + 2, gx.z);
                }
            }
        }
        const float3 acc = f3(A.acc[p]);
        const float3 after = f3(A.Ltot[p]) - acc - Av - Bv;
        if (bits & kAdjTexel) {
            const float4 sa = A.st_a[p];
            const float3 num = delta * (Av + Bv + after);
            double* g = A.g_tex + A.tex_offset[S.materials[mat].albedo_tex] + __float_as_int(sa.w);
            if (sa.x > 0.0f && num.x != 0.0f) atomicAdd(g + 0, double(num.x / sa.x));
            if (sa.y > 0.0f && num.y != 0.0f) atomicAdd(g + 1, double(num.y / sa.y));
            if (sa.z > 0.0f && num.z != 0.0f) atomicAdd(g + 2, double(num.z / sa.z));
        }
        if (bits & kAdjGgx) {
            float gr = 0.0f;
            if (!is_zero(Av)) gr += dot(delta, Av) * sb.x;
            if (!is_zero(Bv)) gr += dot(delta, Bv) * sb.y;
            if (bits & kAdjCont) gr += dot(delta, after) * sb.z;
            adj_add(sh, mat, double(gr));
        }
        const float3 nacc = acc + (Av + Bv);
        A.acc[p] = make_float4(nacc.x, nacc.y, nacc.z, 0.0f);
    }
    adj_shared_flush(sh, A);
}

// Between the two wavefront passes of the adjoint: every path's total
// radiance from the first, and a zero replay accumulator for the second.
__global__ void k_adj_ltot(RenderArgs a) {
    const BatchHeader h = *a.header;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < h.total_paths; p += gridDim.x * blockDim.x) {
        const float3 v = path_sample(f3(a.wf.L[p]), f3(a.wf.Le[p]), f3(a.wf.Ls[p]));
        a.adj.Ltot[p] = make_float4(v.x, v.y, v.z, 0.0f);
        a.adj.acc[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

template <int KIND, bool ADJ = false>
__global__ void k_wf_shade(RenderArgs a, int b) {
    extern __shared__ double adj_sh[];  // ADJ only: gradient block sums
    const WfBuffers& w = a.wf;
    const int n = w.cnt[b * kCntStride + 3 + KIND];
    int* next = w.cnt + (b + 1) * kCntStride;
    const int* q = w.q_mat[KIND];
    const int nb = (b + 1) & 1;
    const uint64_t seed = a.header->seed;
    if (ADJ) adj_shared_zero(adj_sh, a.adj);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = q[i];
        uint4 meta = w.meta[p];
        const SceneD& S = a.scenes[meta.x];
        const float3 o = f3(w.ray_o[p]), d = f3(w.ray_d[p]);
        const float4 h4 = w.hit[p];
        HitD hit;
        hit.t = h4.x;
        hit.slot = __float_as_int(h4.y);
        hit.u = h4.z;
        hit.v = h4.w;
        const SurfaceD si = surface_at(S, o, d, hit);
        const float4 tw = w.thr[p];
        Rng rng;
        rng.key = path_key(seed, meta.x, meta.y, meta.z);
        rng.ctr = meta.w;
        const VertexPlan pl = plan_vertex<KIND>(S, si, f3(tw), (__float_as_int(tw.w) & 1) != 0, b, rng);
        bool adj_live = false;
        if (ADJ) {
            adj_live = adj_vertex_begin(a, adj_sh, S, si, pl, tw, p, meta.y);
        } else if (!is_zero(pl.emit)) {
            float4 L = w.L[p];
            L.x += pl.emit.x;
            L.y += pl.emit.y;
            L.z += pl.emit.z;
            w.L[p] = L;
        }
        // the adjoint drops a path that carries no gradient
        const bool live = !ADJ || adj_live;
        const bool cont = live && pl.cont && (b + 1 < S.max_depth);
        if (pl.shadow || pl.mis || cont) w.ray_o[p] = make_float4(si.P.x, si.P.y, si.P.z, 0.0f);
        if (pl.shadow) {
            w.sh_d[p] = make_float4(pl.sdir.x, pl.sdir.y, pl.sdir.z, pl.stmax);
            w.sh_c[p] = make_float4(pl.scontrib.x, pl.scontrib.y, pl.scontrib.z, 0.0f);
        }
        // only MIS rays that meet their light are traced (mis_light_hit)
        bool mocc = false;
        if (pl.mis && live) {
            float4 mh = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            mocc = mis_light_hit(S, ray_prep(si.P, pl.mdir, kRayEps, kFloatMax), pl.mlight, &mh);
            if (mocc) {
                w.mis_d[p] = make_float4(pl.mdir.x, pl.mdir.y, pl.mdir.z, 0.0f);
                w.mis_a[p] = make_float4(pl.mfactor.x, pl.mfactor.y, pl.mfactor.z, pl.mpdf);
                w.mis_b[p] = make_float4(tw.x, tw.y, tw.z, __int_as_float(pl.mlight));
                w.mis_h[p] = mh;
            }
        }
        if (cont) {
            w.ray_d[p] = make_float4(pl.cdir.x, pl.cdir.y, pl.cdir.z, 0.0f);
            w.thr[p] = make_float4(pl.T.x, pl.T.y, pl.T.z, __int_as_float(pl.count_emission));
        }
        meta.w = rng.ctr;
        w.meta[p] = meta;
        // a shadow ray whose contribution is zero in every channel adds
        // nothing to Ls whatever its outcome (the adjoint still needs it: its
        // radiance derivative need not be zero)
        const int s_slot = warp_append(next + 2, live && pl.shadow != 0 && (ADJ || !is_zero(pl.scontrib)));
        if (s_slot >= 0) w.q_shadow[nb][s_slot] = p;
        const int o_slot = warp_append(next + 11, mocc);
        if (o_slot >= 0) w.q_mocc[nb][o_slot] = p;
        const int c_slot = warp_append(next + 0, cont);
        if (c_slot >= 0) w.q_cont[nb][c_slot] = p;
        if (ADJ) {
            const int v_slot = warp_append(next + 10, adj_live);
            if (v_slot >= 0) a.adj.q_vtx[b & 1][v_slot] = p;
        }
    }
    if (ADJ) adj_shared_flush(adj_sh, a.adj);
}

// FP64 accumulation of one batch into the scenes' films.  With the default
// box filter of size 1 a sample at (ix + fx, iy + fy) lands in pixel (ix, iy)
// only; other filters go through splat_filtered.  NaN / Inf samples are
// dropped as FilmTile::addSample does (source/core/film/filmTile.cpp:21-28).
__global__ void k_splat(RenderArgs a) {
    const BatchHeader h = *a.header;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < h.total_pixels; idx += gridDim.x * blockDim.x) {
        int lo = 0, hi = int(h.num_chunks) - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.chunks[mid].pix_begin <= idx) lo = mid; else hi = mid - 1;
        }
        const Chunk c = a.chunks[lo];
        const uint32_t pixel = idx - c.pix_begin;
        const FilterD& F = a.scenes[c.scene].filter;
        if (!F.pixel_only) {
            double s[3] = {0, 0, 0}, q[3] = {0, 0, 0}, n = 0;
            const int W = int(c.width);
            auto fetch = [&](uint32_t k, int sx, int sy, float3* v, float2* pos) {
                const uint32_t p = c.path_begin + k * c.npix + uint32_t(sy * W + sx);
                const float4 L = a.wf.L[p], Ls = a.wf.Ls[p];
                *v = path_sample(f3(L), f3(a.wf.Le[p]), f3(Ls));
                *pos = make_float2(L.w, Ls.w);
                return isfinite(v->x) && isfinite(v->y) && isfinite(v->z);
            };
            filter_gather(F, W, int(c.npix / c.width), int(pixel % c.width), int(pixel / c.width), c.nsamples, fetch, s,
                          q, &n);
            const FilmD f = a.films[c.scene];
            for (int k = 0; k < 3; ++k) {
                f.sum[3 * pixel + k] += s[k];
                f.sumsq[3 * pixel + k] += q[k];
            }
            f.count[pixel] += n;
            continue;
        }
        double s0 = 0, s1 = 0, s2 = 0, q0 = 0, q1 = 0, q2 = 0, n = 0;
        for (uint32_t k = 0; k < c.nsamples; ++k) {
            const uint32_t p = c.path_begin + k * c.npix + pixel;
            const float3 v = path_sample(f3(a.wf.L[p]), f3(a.wf.Le[p]), f3(a.wf.Ls[p]));
            const float x = v.x, y = v.y, z = v.z;
            if (!(isfinite(x) && isfinite(y) && isfinite(z))) continue;
            s0 += x; s1 += y; s2 += z;
            q0 += double(x) * x; q1 += double(y) * y; q2 += double(z) * z;
            n += 1.0;
        }
        const FilmD f = a.films[c.scene];
        f.sum[3 * pixel + 0] += s0;
        f.sum[3 * pixel + 1] += s1;
        f.sum[3 * pixel + 2] += s2;
        f.sumsq[3 * pixel + 0] += q0;
        f.sumsq[3 * pixel + 1] += q1;
        f.sumsq[3 * pixel + 2] += q2;
        f.count[pixel] += n;
    }
}

__global__ void k_gather_paths(const float4* L, const float4* Le, const float4* Ls, uint32_t n, float* out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const float3 v = path_sample(f3(L[p]), f3(Le[p]), f3(Ls[p]));
        out[3 * p + 0] = v.x;
        out[3 * p + 1] = v.y;
        out[3 * p + 2] = v.z;
    }
}

// ------------------------------------------------------------- ray queries --
__global__ void k_trace(const SceneD* scenes, int scene, const cgpu_ray* rays, uint32_t n, cgpu_hit* hits,
                        uint8_t* occ) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const SceneD& S = scenes[scene];
        const cgpu_ray r = rays[i];
        // the direction is normalised again, as the reference's Ray constructor does (ray.cpp:19-30)
        const RayPre pr = ray_prep(mk(r.org[0], r.org[1], r.org[2]), normalize(mk(r.dir[0], r.dir[1], r.dir[2])),
                                   r.t_min, r.t_max);
        HitD h;
        TraceCounters tc{0, 0};
        if (occ) {
            occ[i] = traverse<true, false>(S, pr, &h, &tc) ? 1 : 0;
        } else {
            cgpu_hit out;
            if (traverse_warp<false>(S, pr, &h, &tc)) {
                const HitPoint hp = hit_point(S, pr.o, pr.d, h);
                out.t = hp.t;
                out.primitive = __float_as_int(ldg4(reinterpret_cast<const float4*>(S.tris + h.slot)).w);
                out.u = hp.rect >= 0 ? hp.p1 : hp.b1;
                out.v = hp.rect >= 0 ? hp.p2 : hp.b2;
            } else {
                out.t = 0.0f;
                out.primitive = -1;
                out.u = 0.0f;
                out.v = 0.0f;
            }
            hits[i] = out;
        }
    }
}

__global__ void k_camera(const SceneD* scenes, int scene, const double* xy, uint32_t n, float* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float3 o, d;
        camera_ray(scenes[scene].cam, float(xy[2 * i]), float(xy[2 * i + 1]), &o, &d);
        out[6 * i + 0] = o.x; out[6 * i + 1] = o.y; out[6 * i + 2] = o.z;
        out[6 * i + 3] = d.x; out[6 * i + 4] = d.y; out[6 * i + 5] = d.z;
    }
}

}  // namespace cg

// ============================================================== host side ==
using namespace cg;

namespace {

constexpr int kBlock = 128;  // fixed-size utility kernels

template <typename K>
int grid_for(cgpu_ctx* ctx, K kernel, int block, uint64_t work, size_t shared_bytes = 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, shared_bytes);
    if (per_sm < 1) per_sm = 1;
    const uint64_t full = uint64_t(ctx->num_sms) * uint64_t(per_sm);
    const uint64_t need = (work + block - 1) / block;
    return int(std::max<uint64_t>(1, std::min<uint64_t>(full, need)));
}

// Dynamic shared memory of a traversal launch: the shared-memory part of the
// traversal stacks of the persistent passes (0 for the other variants).  A
// block above the default 48 KB window opts the kernel in first.
template <typename K>
size_t stack_smem(K kernel, bool shared_stack, bool with_t, int block) {
    if (!shared_stack) return 0;
    const size_t bytes = with_t ? SharedStack<true>::bytes(block) : SharedStack<false>::bytes(block);
    if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
    return bytes;
}

uint32_t paths_capacity(cgpu_ctx* ctx, uint32_t max_npix) {
    uint32_t cap = ctx->tuning.max_paths ? ctx->tuning.max_paths : (1u << 21);
    if (cap < max_npix) cap = max_npix;
    return cap;
}

cgpu_status ensure_path_buffers(cgpu_ctx* ctx, uint32_t cap, int depth) {
    if (ctx->path_cap >= cap && ctx->wf.cnt_depth >= depth + 2) return CGPU_OK;
    cg_free_render_state(ctx);
    const int cdepth = std::max(depth + 2, 34);
    WfBuffers w{};
    const size_t bytes = wf_layout(nullptr, cap, cdepth, &w);
    void* block = nullptr;
    cudaError_t e = cudaMalloc(&block, bytes);
    if (e != cudaSuccess) return cg_fail(ctx, CGPU_ERR_OUT_OF_MEMORY, "path buffers: " + std::string(cudaGetErrorString(e)));
    wf_layout(static_cast<char*>(block), cap, cdepth, &ctx->wf);
    ctx->wf_block = block;
    ctx->path_cap = cap;
    if (!ctx->d_counters) {
        e = cudaMalloc(&ctx->d_counters, 8 * sizeof(unsigned long long));
        if (e != cudaSuccess) return cg_cuda(ctx, e, "counters");
    }
    if (!ctx->d_chunks) {
        if ((e = cudaMalloc(&ctx->d_chunks, sizeof(Chunk) * kMaxChunks)) != cudaSuccess) return cg_cuda(ctx, e, "chunks");
        if ((e = cudaMalloc(&ctx->d_header, sizeof(BatchHeader))) != cudaSuccess) return cg_cuda(ctx, e, "header");
        if ((e = cudaMallocHost(&ctx->h_chunks, sizeof(Chunk) * kMaxChunks)) != cudaSuccess) return cg_cuda(ctx, e, "chunks");
        if ((e = cudaMallocHost(&ctx->h_header, sizeof(BatchHeader))) != cudaSuccess) return cg_cuda(ctx, e, "header");
    }
    return CGPU_OK;
}

uint32_t scan_launches(uint32_t n) {
    const uint32_t nb = radix_tiles(n);
    return 1 + (nb > 1 ? scan_launches(nb) + 1 : 0);
}

// Ray reordering buffers for 2 * path_cap queue entries (continuation + MIS
// rays of a pass), kept while tuning.reorder is on.
cgpu_status ensure_sort_buffers(cgpu_ctx* ctx) {
    if (!ctx->tuning.reorder) return CGPU_OK;
    const uint64_t cap = uint64_t(ctx->path_cap) * 2;
    if (ctx->sort_block && ctx->sort_cap >= cap) return CGPU_OK;
    if (ctx->sort_block) cudaFree(ctx->sort_block);
    ctx->sort_block = nullptr;
    ctx->sort_cap = 0;
    const uint32_t tiles = radix_tiles(cap);
    const size_t words[] = {cap, cap, cap, cap, size_t(tiles) * 256, scan_scratch(uint64_t(tiles) * 256), 1};
    size_t total = 0;
    for (size_t w : words) total += (w * sizeof(uint32_t) + 255) & ~size_t(255);
    cudaError_t e = cudaMalloc(&ctx->sort_block, total);
    if (e != cudaSuccess) {
        ctx->sort_block = nullptr;
        return cg_fail(ctx, CGPU_ERR_OUT_OF_MEMORY, "reorder buffers: " + std::string(cudaGetErrorString(e)));
    }
    uint32_t* ptr[7];
    char* base = static_cast<char*>(ctx->sort_block);
    for (int i = 0; i < 7; ++i) {
        ptr[i] = reinterpret_cast<uint32_t*>(base);
        base += (words[i] * sizeof(uint32_t) + 255) & ~size_t(255);
    }
    ctx->sort = SortBufs{{ptr[0], ptr[1]}, {ptr[2], ptr[3]}, ptr[4], ptr[5], ptr[6], tiles};
    ctx->sort_cap = uint32_t(cap);
    return CGPU_OK;
}

RenderArgs make_args(cgpu_ctx* ctx) {
    RenderArgs a{};
    a.scenes = ctx->d_scenes;
    a.chunks = ctx->d_chunks;
    a.header = ctx->d_header;
    a.films = ctx->d_films;
    a.wf = ctx->wf;
    a.counters = ctx->d_counters;
    a.adj = AdjBufs{};
    a.sorted = nullptr;
    a.refill_closest = refill_lanes(ctx->tuning.refill_closest);
    a.refill_any = refill_lanes(ctx->tuning.refill_any);
    return a;
}

// Launch wrapper: with profiling on, bracket the launch with CUDA events on
// the stream it runs on.
template <typename F>
void timed(cgpu_ctx* ctx, int cls, cudaStream_t s, F&& launch) {
    if (!ctx->profiling) {
        launch();
        return;
    }
    cgpu_ctx::ProfEvent ev{cls, nullptr, nullptr};
    cudaEventCreate(&ev.a);
    cudaEventCreate(&ev.b);
    cudaEventRecord(ev.a, s);
    launch();
    cudaEventRecord(ev.b, s);
    ctx->prof.push_back(ev);
}

void collect_profile(cgpu_ctx* ctx) {
    if (ctx->prof.empty()) return;
    cudaDeviceSynchronize();
    for (auto& ev : ctx->prof) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev.a, ev.b);
        ctx->times.ms[ev.cls] += ms;
        ctx->times.launches[ev.cls] += 1;
        cudaEventDestroy(ev.a);
        cudaEventDestroy(ev.b);
    }
    ctx->prof.clear();
}

// Enqueue the wavefront schedule for one batch on ctx->stream.
cgpu_status enqueue_wavefront(cgpu_ctx* ctx, int depth, uint32_t paths, bool splat, bool counting) {
    RenderArgs a = make_args(ctx);
    // With per-kernel timing on, the shadow pass runs after the extend pass on
    // the same stream, so that each event pair brackets one kernel alone.
    cudaStream_t s = ctx->stream, side = ctx->profiling ? ctx->stream : ctx->side;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    cudaMemsetAsync(ctx->wf.cnt, 0, size_t(depth + 2) * kCntStride * sizeof(int), s);
    uint32_t launches = 1;
    const int bt = ctx->tuning.block_trace, bs = ctx->tuning.block_shade;
    const int ggen = grid_for(ctx, k_wf_generate, kBlock, paths);
    timed(ctx, CGPU_KERNEL_GENERATE, s, [&] { k_wf_generate<<<ggen, kBlock, 0, s>>>(a); });
    const int trav = ctx->tuning.traversal;
    const bool sph = ctx->batch_spheres;
#define CG_PICK(K) (sph ? (counting ? K<true, true> : K<false, true>) : (counting ? K<true, false> : K<false, false>))
    auto ext_kernel = trav == 1 ? CG_PICK(k_wf_extend_dyn)
                      : (trav == 2 || trav == 3) ? CG_PICK(k_wf_extend_pww) : CG_PICK(k_wf_extend);
    auto sh_kernel = trav == 1 ? CG_PICK(k_wf_shadow_dyn) : trav == 3 ? CG_PICK(k_wf_shadow_pww) : CG_PICK(k_wf_shadow);
    auto mocc_kernel = CG_PICK(k_wf_mis_occl);
    auto ties_kernel = CG_PICK(k_wf_ties);
#undef CG_PICK
    // reordered closest-hit passes after the first (the primary rays are in pixel order already)
    const bool reorder = ctx->tuning.reorder != 0 && trav != 1 && ctx->sort_block != nullptr;
#define CG_PICK_SORTED(C, S) (trav >= 2 ? k_wf_extend_pww<C, S, true> : k_wf_extend<C, S, false, true>)
    auto ext_sorted = sph ? (counting ? CG_PICK_SORTED(true, true) : CG_PICK_SORTED(false, true))
                          : (counting ? CG_PICK_SORTED(true, false) : CG_PICK_SORTED(false, false));
#undef CG_PICK_SORTED
    // reorder 1 / 2 / 3 / 4: 9 / 7 / 4 / 0 Morton bits per axis, 4 / 3 / 2 / 1 sort passes of 8 bits
    // (4: the direction octant alone); an odd pass count leaves the sorted values in the second buffer
    const int sort_bits = ctx->tuning.reorder == 1 ? 9 : ctx->tuning.reorder == 2 ? 7 : ctx->tuning.reorder == 3 ? 4 : 0;
    const int sort_passes = (3 + 3 * sort_bits + 7) / 8;
    if (reorder) a.sorted = ctx->sort.vals[sort_passes & 1];
    const int gkeys = grid_for(ctx, k_ray_keys, 256, uint64_t(paths) * 2);
    // the persistent passes keep the bottom of their traversal stacks in shared memory
    const size_t ext_sm = stack_smem(ext_kernel, trav >= 2, true, bt);
    const size_t ext_sorted_sm = stack_smem(ext_sorted, trav >= 2, true, bt);
    const size_t sh_sm = stack_smem(sh_kernel, trav == 3, false, bt);
    const int gext = grid_for(ctx, ext_kernel, bt, paths, ext_sm);
    const int gsh = grid_for(ctx, sh_kernel, bt, paths, sh_sm);
    const int gmo = grid_for(ctx, mocc_kernel, bt, paths);
    const int gties = grid_for(ctx, ties_kernel, kTieBlock, paths);
    const int gsd[kNumBsdfKinds] = {grid_for(ctx, k_wf_shade<0>, bs, paths), grid_for(ctx, k_wf_shade<1>, bs, paths),
                                    grid_for(ctx, k_wf_shade<2>, bs, paths), grid_for(ctx, k_wf_shade<3>, bs, paths),
                                    grid_for(ctx, k_wf_shade<4>, bs, paths)};
    for (int b = 0; b <= depth; ++b) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
        if (reorder && b > 0) {
            const SortBufs& q = ctx->sort;
            timed(ctx, CGPU_KERNEL_REORDER, s, [&] {
                k_ray_keys<<<gkeys, 256, 0, s>>>(a, b, sort_bits, q.keys[0], q.vals[0], q.n);
                radix_sort_pairs<uint32_t>(q.keys, q.vals, 0, q.n, q.tiles, sort_passes, q.hist, q.sums, s);
            });
            launches += 1 + sort_passes * (2 + scan_launches(q.tiles * 256));
            timed(ctx, CGPU_KERNEL_EXTEND, s, [&] { ext_sorted<<<gext, bt, ext_sorted_sm, s>>>(a, b); });
        } else {
            timed(ctx, CGPU_KERNEL_EXTEND, s, [&] { ext_kernel<<<gext, bt, ext_sm, s>>>(a, b); });
        }
        if (trav >= 2) {
            // the persistent pass's rays within the tie window
            timed(ctx, CGPU_KERNEL_TIES, s, [&] { ties_kernel<<<gties, kTieBlock, 0, s>>>(a, b); });
            launches += 1;
        }
        timed(ctx, CGPU_KERNEL_SHADOW, side, [&] { sh_kernel<<<gsh, bt, sh_sm, side>>>(a, b); });
        // the MIS rays of the vertices of bounce b - 1 that meet their light
        if (b > 0) {
            timed(ctx, CGPU_KERNEL_MIS_OCCL, side, [&] { mocc_kernel<<<gmo, bt, 0, side>>>(a, b); });
            launches += 1;
        }
        cudaEventRecord(join, side);
        cudaStreamWaitEvent(s, join, 0);
        launches += 2;
        if (b == depth) break;
        timed(ctx, CGPU_KERNEL_SHADE, s, [&] {
            k_wf_shade<0><<<gsd[0], bs, 0, s>>>(a, b);
            k_wf_shade<1><<<gsd[1], bs, 0, s>>>(a, b);
            k_wf_shade<2><<<gsd[2], bs, 0, s>>>(a, b);
            k_wf_shade<3><<<gsd[3], bs, 0, s>>>(a, b);
            k_wf_shade<4><<<gsd[4], bs, 0, s>>>(a, b);
        });
        launches += kNumBsdfKinds;
    }
    if (splat) {
        const int gsp = grid_for(ctx, k_splat, 256, ctx->h_header->total_pixels);
        timed(ctx, CGPU_KERNEL_SPLAT, s, [&] { k_splat<<<gsp, 256, 0, s>>>(a); });
        launches += 1;
    }
    cudaEventDestroy(fork);
    cudaEventDestroy(join);
    ctx->stats.kernel_launches += launches;
    return cg_cuda(ctx, cudaGetLastError(), "wavefront launch");
}

cgpu_status run_batch(cgpu_ctx* ctx, int mode, int depth, uint32_t paths, bool splat, bool use_graph) {
    const bool counting = ctx->counting;
    if (mode == CGPU_MODE_MEGAKERNEL) {
        RenderArgs a = make_args(ctx);
        const int bt = ctx->tuning.block_trace;
        const bool sph = ctx->batch_spheres;
        if (counting) {
            auto k = sph ? k_megakernel<true, true> : k_megakernel<true, false>;
            k<<<grid_for(ctx, k, bt, paths), bt, 0, ctx->stream>>>(a);
        } else {
            auto k = sph ? k_megakernel<false, true> : k_megakernel<false, false>;
            const int g = grid_for(ctx, k, bt, paths);
            timed(ctx, CGPU_KERNEL_MEGAKERNEL, ctx->stream, [&] { k<<<g, bt, 0, ctx->stream>>>(a); });
        }
        ctx->stats.kernel_launches += 1;
        if (splat) {
            const int gsp = grid_for(ctx, k_splat, 256, ctx->h_header->total_pixels);
            timed(ctx, CGPU_KERNEL_SPLAT, ctx->stream, [&] { k_splat<<<gsp, 256, 0, ctx->stream>>>(a); });
            ctx->stats.kernel_launches += 1;
        }
        return cg_cuda(ctx, cudaGetLastError(), "megakernel launch");
    }
    if (!use_graph || counting || !splat || ctx->profiling) return enqueue_wavefront(ctx, depth, paths, splat, counting);
    // one graph per (depth, path capacity, sphere kernels); the batch itself lives in device memory
    if (!ctx->graph || ctx->graph_depth != depth || ctx->graph_paths != ctx->path_cap ||
        ctx->graph_spheres != ctx->batch_spheres) {
        if (ctx->graph) {
            cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "begin capture");
        const uint32_t before = ctx->stats.kernel_launches;
        // capture for the full capacity: kernels read the live path count from the header
        cgpu_status st = enqueue_wavefront(ctx, depth, ctx->path_cap, true, false);
        e = cudaStreamEndCapture(ctx->stream, &g);
        if (st != CGPU_OK) return st;
        if (e != cudaSuccess) return cg_cuda(ctx, e, "end capture");
        e = cudaGraphInstantiate(&ctx->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "graph instantiate");
        ctx->graph_depth = depth;
        ctx->graph_paths = ctx->path_cap;
        ctx->graph_spheres = ctx->batch_spheres;
        ctx->graph_launches = ctx->stats.kernel_launches - before;
        ctx->stats.kernel_launches = before;
    }
    ctx->stats.kernel_launches += ctx->graph_launches;
    return cg_cuda(ctx, cudaGraphLaunch(ctx->graph, ctx->stream), "graph launch");
}

}  // namespace

void cg_free_render_state(cgpu_ctx* ctx) {
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    ctx->graph_depth = -1;
    if (ctx->wf_block) {
        cudaFree(ctx->wf_block);
        ctx->wf_block = nullptr;
    }
    ctx->wf = WfBuffers{};
    ctx->path_cap = 0;
    if (ctx->adj_block) {
        cudaFree(ctx->adj_block);
        ctx->adj_block = nullptr;
    }
    ctx->adj = AdjBufs{};
    ctx->adj_cap = 0;
    if (ctx->sort_block) {
        cudaFree(ctx->sort_block);
        ctx->sort_block = nullptr;
    }
    ctx->sort = SortBufs{};
    ctx->sort_cap = 0;
}

// Split the requested samples of every scene into batches of at most
// path_cap paths and run them.
cgpu_status cg_render_batches(cgpu_ctx* ctx, const cgpu_render_params* p) {
    if (!p || !p->scenes || p->num_scenes == 0 || p->num_scenes > uint32_t(kMaxChunks))
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render: bad scene list");
    if (p->mode != CGPU_MODE_MEGAKERNEL && p->mode != CGPU_MODE_WAVEFRONT)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render: unknown mode");
    uint32_t max_npix = 0;
    int depth = 1;
    for (uint32_t i = 0; i < p->num_scenes; ++i) {
        const int s = p->scenes[i];
        if (s < 0 || s >= int(ctx->scenes.size()) || !ctx->scenes[s].live)
            return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "render: unknown scene id");
        const SceneSlot& sl = ctx->scenes[s];
        max_npix = std::max<uint32_t>(max_npix, uint32_t(sl.width) * uint32_t(sl.height));
        depth = std::max(depth, sl.max_depth);
    }
    bool spheres = false;
    for (uint32_t i = 0; i < p->num_scenes; ++i) spheres |= ctx->scenes[p->scenes[i]].has_spheres;
    ctx->batch_spheres = spheres;
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    st = ensure_path_buffers(ctx, paths_capacity(ctx, max_npix), depth);
    if (st != CGPU_OK) return st;
    st = ensure_sort_buffers(ctx);
    if (st != CGPU_OK) return st;
    ctx->stats = cgpu_render_stats{};
    ctx->times = cgpu_kernel_times{};
    if (ctx->counting) cudaMemsetAsync(ctx->d_counters, 0, 8 * sizeof(unsigned long long), ctx->stream);
    // remaining samples per scene
    std::vector<uint32_t> next(p->num_scenes, p->first_sample), end(p->num_scenes);
    for (uint32_t i = 0; i < p->num_scenes; ++i) {
        const uint64_t n = p->scene_samples ? p->scene_samples[i] : p->num_samples;
        if (uint64_t(p->first_sample) + n > 0xFFFFFFFFull)
            return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render: sample range overflows 32 bits");
        end[i] = p->first_sample + uint32_t(n);
    }
    uint64_t total_paths = 0;
    for (;;) {
        uint32_t used = 0, pix = 0, nch = 0;
        for (uint32_t i = 0; i < p->num_scenes && nch < uint32_t(kMaxChunks); ++i) {
            if (next[i] >= end[i]) continue;
            const SceneSlot& sl = ctx->scenes[p->scenes[i]];
            const uint32_t npix = uint32_t(sl.width) * uint32_t(sl.height);
            const uint32_t room = (ctx->path_cap - used) / npix;
            if (room == 0) continue;
            const uint32_t k = std::min(room, end[i] - next[i]);
            Chunk& c = ctx->h_chunks[nch++];
            c.scene = p->scenes[i];
            c.path_begin = used;
            c.npix = npix;
            c.width = uint32_t(sl.width);
            c.sample0 = next[i];
            c.nsamples = k;
            c.pix_begin = pix;
            c.pad = 0;
            used += k * npix;
            pix += npix;
            next[i] += k;
        }
        if (nch == 0) break;
        BatchHeader& h = *ctx->h_header;
        // the previous batch may still read the pinned staging copies
        cudaStreamSynchronize(ctx->stream);
        h.num_chunks = nch;
        h.total_paths = used;
        h.total_pixels = pix;
        h.max_depth = depth;
        h.seed = p->seed;
        cudaMemcpyAsync(ctx->d_chunks, ctx->h_chunks, sizeof(Chunk) * nch, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(ctx->d_header, ctx->h_header, sizeof(BatchHeader), cudaMemcpyHostToDevice, ctx->stream);
        st = run_batch(ctx, p->mode, depth, used, true, p->use_graph != 0);
        if (st != CGPU_OK) return st;
        total_paths += used;
        ctx->stats.batches += 1;
        ctx->stats.h2d_bytes += sizeof(Chunk) * nch + sizeof(BatchHeader);
        collect_profile(ctx);
    }
    ctx->stats.paths = total_paths;
    if (ctx->counting) {
        unsigned long long c[8];
        cudaMemcpyAsync(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        ctx->stats.closest_rays = c[0];
        ctx->stats.any_rays = c[1];
        ctx->stats.node_visits = c[2];
        ctx->stats.triangle_tests = c[3];
        ctx->stats.any_node_visits = c[4];
        ctx->stats.any_triangle_tests = c[5];
        ctx->stats.tie_rays = c[6];
    }
    return cg_cuda(ctx, cudaGetLastError(), "render");
}

cgpu_status cg_render_paths_raw(cgpu_ctx* ctx, int scene, int mode, uint32_t first, uint32_t count, uint64_t seed,
                                float* host_rgb) {
    if (scene < 0 || scene >= int(ctx->scenes.size()) || !ctx->scenes[scene].live)
        return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "render_paths: unknown scene id");
    const SceneSlot& sl = ctx->scenes[scene];
    const uint32_t npix = uint32_t(sl.width) * uint32_t(sl.height);
    ctx->batch_spheres = sl.has_spheres;
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    st = ensure_path_buffers(ctx, paths_capacity(ctx, npix), sl.max_depth);
    if (st != CGPU_OK) return st;
    st = ensure_sort_buffers(ctx);
    if (st != CGPU_OK) return st;
    float* d_out = nullptr;
    const uint32_t per = std::max<uint32_t>(1, ctx->path_cap / npix);
    cudaError_t e = cudaMalloc(&d_out, size_t(per) * npix * 3 * sizeof(float));
    if (e != cudaSuccess) return cg_cuda(ctx, e, "render_paths buffer");
    for (uint32_t done = 0; done < count;) {
        const uint32_t k = std::min(per, count - done);
        cudaStreamSynchronize(ctx->stream);
        Chunk& c = ctx->h_chunks[0];
        c = Chunk{scene, 0, npix, uint32_t(sl.width), first + done, k, 0, 0};
        BatchHeader& h = *ctx->h_header;
        h.num_chunks = 1;
        h.total_paths = k * npix;
        h.total_pixels = npix;
        h.max_depth = sl.max_depth;
        h.seed = seed;
        cudaMemcpyAsync(ctx->d_chunks, ctx->h_chunks, sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(ctx->d_header, ctx->h_header, sizeof(BatchHeader), cudaMemcpyHostToDevice, ctx->stream);
        st = run_batch(ctx, mode, sl.max_depth, k * npix, false, false);
        if (st != CGPU_OK) break;
        k_gather_paths<<<grid_for(ctx, k_gather_paths, 256, k * npix), 256, 0, ctx->stream>>>(ctx->wf.L, ctx->wf.Le, ctx->wf.Ls, k * npix, d_out);
        cudaMemcpyAsync(host_rgb + size_t(done) * npix * 3, d_out, size_t(k) * npix * 3 * sizeof(float),
                        cudaMemcpyDeviceToHost, ctx->stream);
        done += k;
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_out);
    if (st != CGPU_OK) return st;
    return cg_cuda(ctx, cudaGetLastError(), "render_paths");
}

cgpu_status cg_path_radiance(cgpu_ctx* ctx, int scene, int mode, const double* film_xy, const uint64_t* keys,
                             uint32_t n, float* out_rgb) {
    (void)mode;  // one path per thread either way: both modes share plan_vertex / resolve
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    double* d_xy = nullptr;
    uint64_t* d_keys = nullptr;
    float* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_xy, size_t(n) * 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_keys, size_t(n) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, size_t(n) * 12);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_xy, film_xy, size_t(n) * 16, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_keys, keys, size_t(n) * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        k_paths_explicit<<<grid_for(ctx, k_paths_explicit, kBlock, n), kBlock, 0, ctx->stream>>>(ctx->d_scenes, scene, d_xy,
                                                                                                d_keys, n, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_rgb, d_out, size_t(n) * 12, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_xy);
    cudaFree(d_keys);
    cudaFree(d_out);
    return cg_cuda(ctx, e, "path_radiance");
}

cgpu_status cg_trace(cgpu_ctx* ctx, int scene, const cgpu_ray* d_rays, uint32_t n, cgpu_hit* d_hits, uint8_t* d_occ,
                     bool any) {
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    if (n == 0) return CGPU_OK;
    k_trace<<<grid_for(ctx, k_trace, kBlock, n), kBlock, 0, ctx->stream>>>(ctx->d_scenes, scene, d_rays, n,
                                                                        any ? nullptr : d_hits, any ? d_occ : nullptr);
    return cg_cuda(ctx, cudaGetLastError(), "trace launch");
}

cgpu_status cg_camera(cgpu_ctx* ctx, int scene, const double* d_xy, uint32_t n, float* d_out) {
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    if (n == 0) return CGPU_OK;
    k_camera<<<grid_for(ctx, k_camera, kBlock, n), kBlock, 0, ctx->stream>>>(ctx->d_scenes, scene, d_xy, n, d_out);
    return cg_cuda(ctx, cudaGetLastError(), "camera launch");
}

cgpu_status cg_film_clear(cgpu_ctx* ctx, int scene) {
    SceneSlot& sl = ctx->scenes[scene];
    const size_t npix = size_t(sl.width) * sl.height;
    cudaMemsetAsync(sl.film.sum, 0, npix * 3 * sizeof(double), ctx->stream);
    cudaMemsetAsync(sl.film.sumsq, 0, npix * 3 * sizeof(double), ctx->stream);
    cudaMemsetAsync(sl.film.count, 0, npix * sizeof(double), ctx->stream);
    return cg_cuda(ctx, cudaGetLastError(), "film clear");
}

// ======================================================= wavefront adjoint ==
// cgpu_adjoint_backward on the wavefront schedule.  Per batch of whole
// samples of the scene: (A) the forward wavefront render of the batch without
// the film splat, whose per-path radiance is the Ltot of each path; (B) the
// same paths regenerated and replayed pass by pass with the adjoint variants
// of the kernels (extend / shadow store the MIS and shadow outcomes instead of
// adding them; shade keeps each vertex's state and queues it), and after each
// traversal pass the gradient kernel of the vertices whose rays it traced.
namespace {

void enqueue_adjoint_pass(cgpu_ctx* ctx, const RenderArgs& a, int depth, uint32_t paths, size_t shared_bytes) {
    cudaStream_t s = ctx->stream, side = ctx->side;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    cudaMemsetAsync(ctx->wf.cnt, 0, size_t(depth + 2) * kCntStride * sizeof(int), s);
    const int bt = ctx->tuning.block_trace, bs = ctx->tuning.block_shade;
    const bool sph = ctx->batch_spheres;
    // the persistent passes when the tuning uses them (traversal 2 / 3), else the per-ray loops
    const int trav = ctx->tuning.traversal;
    auto ext = trav >= 2 ? (sph ? k_wf_extend_pww<false, true, false, true> : k_wf_extend_pww<false, false, false, true>)
                         : (sph ? k_wf_extend<false, true, true> : k_wf_extend<false, false, true>);
    auto shd = trav == 3 ? (sph ? k_wf_shadow_pww<false, true, true> : k_wf_shadow_pww<false, false, true>)
                         : (sph ? k_wf_shadow<false, true, true> : k_wf_shadow<false, false, true>);
    auto mo = sph ? k_wf_mis_occl<false, true, true> : k_wf_mis_occl<false, false, true>;
    auto ties = sph ? k_wf_ties<false, true, true> : k_wf_ties<false, false, true>;
    void (*shade[kNumBsdfKinds])(RenderArgs, int) = {k_wf_shade<0, true>, k_wf_shade<1, true>, k_wf_shade<2, true>,
                                                     k_wf_shade<3, true>, k_wf_shade<4, true>};
    k_wf_generate<<<grid_for(ctx, k_wf_generate, kBlock, paths), kBlock, 0, s>>>(a);
    const size_t ext_sm = stack_smem(ext, trav >= 2, true, bt), sh_sm = stack_smem(shd, trav == 3, false, bt);
    const int gext = grid_for(ctx, ext, bt, paths, ext_sm), gsh = grid_for(ctx, shd, bt, paths, sh_sm);
    const int gmo = grid_for(ctx, mo, bt, paths), gties = grid_for(ctx, ties, kTieBlock, paths);
    const int gv = grid_for(ctx, k_adj_vertex, kBlock, paths, shared_bytes);
    int gsd[kNumBsdfKinds];
    for (int k = 0; k < kNumBsdfKinds; ++k) gsd[k] = grid_for(ctx, shade[k], bs, paths, shared_bytes);
    uint32_t launches = 1;
    for (int b = 0; b <= depth; ++b) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
        ext<<<gext, bt, ext_sm, s>>>(a, b);
        if (trav >= 2) {
            ties<<<gties, kTieBlock, 0, s>>>(a, b);
            launches += 1;
        }
        shd<<<gsh, bt, sh_sm, side>>>(a, b);
        if (b > 0) {
            mo<<<gmo, bt, 0, side>>>(a, b);
            launches += 1;
        }
        cudaEventRecord(join, side);
        cudaStreamWaitEvent(s, join, 0);
        launches += 2;
        if (b > 0) {
            k_adj_vertex<<<gv, kBlock, shared_bytes, s>>>(a, b - 1);
            launches += 1;
        }
        if (b == depth) break;
        for (int k = 0; k < kNumBsdfKinds; ++k) shade[k]<<<gsd[k], bs, shared_bytes, s>>>(a, b);
        launches += kNumBsdfKinds;
    }
    cudaEventDestroy(fork);
    cudaEventDestroy(join);
    ctx->stats.kernel_launches += launches;
}

cgpu_status ensure_adj_buffers(cgpu_ctx* ctx) {
    if (ctx->adj_cap >= ctx->path_cap && ctx->adj_block) return CGPU_OK;
    if (ctx->adj_block) cudaFree(ctx->adj_block);
    ctx->adj_block = nullptr;
    ctx->adj_cap = 0;
    AdjBufs tmp{};
    const size_t bytes = adj_layout(nullptr, ctx->path_cap, &tmp);
    cudaError_t e = cudaMalloc(&ctx->adj_block, bytes);
    if (e != cudaSuccess) {
        ctx->adj_block = nullptr;
        return cg_fail(ctx, CGPU_ERR_OUT_OF_MEMORY, "adjoint buffers: " + std::string(cudaGetErrorString(e)));
    }
    adj_layout(static_cast<char*>(ctx->adj_block), ctx->path_cap, &ctx->adj);
    ctx->adj_cap = ctx->path_cap;
    return CGPU_OK;
}

}  // namespace

cgpu_status cg_adjoint_wavefront(cgpu_ctx* ctx, int scene, uint32_t spp, uint64_t seed, const AdjBufs& params) {
    const SceneSlot& sl = ctx->scenes[scene];
    const uint32_t npix = uint32_t(sl.width) * uint32_t(sl.height);
    ctx->batch_spheres = sl.has_spheres;
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    st = ensure_path_buffers(ctx, paths_capacity(ctx, npix), sl.max_depth);
    if (st != CGPU_OK) return st;
    st = ensure_adj_buffers(ctx);
    if (st != CGPU_OK) return st;
    const size_t shared_bytes = size_t(params.nmat + 3 * params.nlight) * sizeof(double);
    if (shared_bytes > 48 * 1024) {
        const int sb = int(shared_bytes);
        cudaFuncSetAttribute(k_adj_vertex, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
        cudaFuncSetAttribute(k_wf_shade<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
        cudaFuncSetAttribute(k_wf_shade<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
        cudaFuncSetAttribute(k_wf_shade<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
        cudaFuncSetAttribute(k_wf_shade<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
        cudaFuncSetAttribute(k_wf_shade<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
    }
    RenderArgs a = make_args(ctx);
    a.adj = params;
    a.adj.Ltot = ctx->adj.Ltot;
    a.adj.acc = ctx->adj.acc;
    a.adj.st_a = ctx->adj.st_a;
    a.adj.st_b = ctx->adj.st_b;
    a.adj.st_c = ctx->adj.st_c;
    a.adj.mis_B = ctx->adj.mis_B;
    a.adj.mis_X = ctx->adj.mis_X;
    a.adj.q_vtx[0] = ctx->adj.q_vtx[0];
    a.adj.q_vtx[1] = ctx->adj.q_vtx[1];
    ctx->stats = cgpu_render_stats{};
    const uint32_t per = std::max<uint32_t>(1, ctx->path_cap / npix);
    const int depth = sl.max_depth;
    for (uint32_t done = 0; done < spp;) {
        const uint32_t k = std::min(per, spp - done);
        const uint32_t paths = k * npix;
        cudaStreamSynchronize(ctx->stream);
        ctx->h_chunks[0] = Chunk{scene, 0, npix, uint32_t(sl.width), done, k, 0, 0};
        BatchHeader& h = *ctx->h_header;
        h.num_chunks = 1;
        h.total_paths = paths;
        h.total_pixels = npix;
        h.max_depth = depth;
        h.seed = seed;
        cudaMemcpyAsync(ctx->d_chunks, ctx->h_chunks, sizeof(Chunk), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(ctx->d_header, ctx->h_header, sizeof(BatchHeader), cudaMemcpyHostToDevice, ctx->stream);
        st = enqueue_wavefront(ctx, depth, paths, false, false);
        if (st != CGPU_OK) return st;
        k_adj_ltot<<<grid_for(ctx, k_adj_ltot, 256, paths), 256, 0, ctx->stream>>>(a);
        ctx->stats.kernel_launches += 1;
        enqueue_adjoint_pass(ctx, a, depth, paths, shared_bytes);
        st = cg_cuda(ctx, cudaGetLastError(), "adjoint wavefront launch");
        if (st != CGPU_OK) return st;
        ctx->stats.batches += 1;
        done += k;
    }
    ctx->stats.paths = uint64_t(spp) * npix;
    collect_profile(ctx);  // the forward passes' events, with profiling on
    return CGPU_OK;
}

// =========================================================== no-alloc render ==
// cgpu_render_noalloc: the wavefront render of one scene with every device
// buffer the call needs in a static array of this library, so that the call
// itself allocates nothing.  Same kernels as cgpu_render; the batch tables are
// written by a one-block setup kernel (arguments by value, no copies), the
// traversal passes run one after the other on the context stream (no side
// stream, no events, no graph).

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace cg {

// Writes the batch tables and zeroes the queue counters of one batch.
__global__ void k_noalloc_setup(NoAllocView v, BatchHeader h, Chunk c, SceneD sd, FilmD fd, int scene, int cnt_ints) {
    for (int i = threadIdx.x; i < cnt_ints; i += blockDim.x) v.wf.cnt[i] = 0;
    if (threadIdx.x == 0) {
        *v.header = h;
        *v.chunk = c;
        v.scenes[scene] = sd;
        v.films[scene] = fd;
    }
}

}  // namespace cg

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
char* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of the scratch, looked up once per device (the caller has
// made ctx->device current).
cgpu_status noalloc_base(cgpu_ctx* ctx, char** out) {
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    char*& p = g_noalloc_base[ctx->device];
    if (!p) {
        void* a = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "render_noalloc: scratch address");
        p = static_cast<char*>(a);
    }
    *out = p;
    return CGPU_OK;
}

void enqueue_wavefront_serial(cgpu_ctx* ctx, const RenderArgs& a, int depth, uint32_t paths, uint32_t npix) {
    cudaStream_t s = ctx->stream;
    const int bt = ctx->tuning.block_trace, bs = ctx->tuning.block_shade;
    const int trav = ctx->tuning.traversal;
    const bool sph = ctx->batch_spheres;
    auto ext = trav == 1   ? (sph ? k_wf_extend_dyn<false, true> : k_wf_extend_dyn<false, false>)
               : trav >= 2 ? (sph ? k_wf_extend_pww<false, true> : k_wf_extend_pww<false, false>)
                           : (sph ? k_wf_extend<false, true> : k_wf_extend<false, false>);
    auto sh = trav == 1   ? (sph ? k_wf_shadow_dyn<false, true> : k_wf_shadow_dyn<false, false>)
              : trav == 3 ? (sph ? k_wf_shadow_pww<false, true> : k_wf_shadow_pww<false, false>)
                          : (sph ? k_wf_shadow<false, true> : k_wf_shadow<false, false>);
    k_wf_generate<<<grid_for(ctx, k_wf_generate, kBlock, paths), kBlock, 0, s>>>(a);
    const size_t ext_sm = stack_smem(ext, trav >= 2, true, bt), sh_sm = stack_smem(sh, trav == 3, false, bt);
    const int gext = grid_for(ctx, ext, bt, paths, ext_sm), gsh = grid_for(ctx, sh, bt, paths, sh_sm);
    const int gsd[kNumBsdfKinds] = {grid_for(ctx, k_wf_shade<0>, bs, paths), grid_for(ctx, k_wf_shade<1>, bs, paths),
                                    grid_for(ctx, k_wf_shade<2>, bs, paths), grid_for(ctx, k_wf_shade<3>, bs, paths),
                                    grid_for(ctx, k_wf_shade<4>, bs, paths)};
    auto mocc = sph ? k_wf_mis_occl<false, true> : k_wf_mis_occl<false, false>;
    auto ties = sph ? k_wf_ties<false, true> : k_wf_ties<false, false>;
    const int gmo = grid_for(ctx, mocc, bt, paths);
    const int gties = grid_for(ctx, ties, kTieBlock, paths);
    for (int b = 0; b <= depth; ++b) {
        ext<<<gext, bt, ext_sm, s>>>(a, b);
        if (trav >= 2) ties<<<gties, kTieBlock, 0, s>>>(a, b);
        sh<<<gsh, bt, sh_sm, s>>>(a, b);
        if (b > 0) mocc<<<gmo, bt, 0, s>>>(a, b);
        if (b == depth) break;
        k_wf_shade<0><<<gsd[0], bs, 0, s>>>(a, b);
        k_wf_shade<1><<<gsd[1], bs, 0, s>>>(a, b);
        k_wf_shade<2><<<gsd[2], bs, 0, s>>>(a, b);
        k_wf_shade<3><<<gsd[3], bs, 0, s>>>(a, b);
        k_wf_shade<4><<<gsd[4], bs, 0, s>>>(a, b);
    }
    k_splat<<<grid_for(ctx, k_splat, 256, npix), 256, 0, s>>>(a);
    ctx->stats.kernel_launches +=
        uint32_t(3 + 2 * (depth + 1) + depth + kNumBsdfKinds * depth + (trav >= 2 ? depth + 1 : 0));
}

}  // namespace

extern "C" cgpu_status cgpu_render_noalloc(cgpu_ctx* ctx, int32_t scene, uint32_t first_sample, uint32_t num_samples,
                                           uint64_t seed) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (scene < 0 || scene >= int32_t(ctx->scenes.size()) || !ctx->scenes[size_t(scene)].live)
        return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "render_noalloc: unknown scene id");
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    const uint64_t npix = uint64_t(sl.width) * uint64_t(sl.height);
    if (scene >= kNoAllocMaxScenes)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_noalloc: scene id " + std::to_string(scene) +
                                                           " is not below the static scratch's " +
                                                           std::to_string(kNoAllocMaxScenes) + " scene slots");
    if (npix > kNoAllocMaxPaths)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_noalloc: " + std::to_string(sl.width) + " x " +
                                                           std::to_string(sl.height) + " pixels exceed the " +
                                                           std::to_string(kNoAllocMaxPaths) +
                                                           " paths of the static scratch");
    if (sl.max_depth > kNoAllocMaxDepth)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_noalloc: max depth " + std::to_string(sl.max_depth) +
                                                           " exceeds " + std::to_string(kNoAllocMaxDepth));
    if (uint64_t(first_sample) + num_samples > 0xFFFFFFFFull)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_noalloc: sample range overflows 32 bits");
    if (num_samples == 0) return CGPU_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cg_cuda(ctx, e, "render_noalloc: set device");
    char* base = nullptr;
    cgpu_status st = noalloc_base(ctx, &base);
    if (st != CGPU_OK) return st;
    NoAllocView v;
    if (noalloc_layout(base, &v) > kNoAllocScratchBytes)
        return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "render_noalloc: scratch layout exceeds the static array");
    RenderArgs a{};
    a.scenes = v.scenes;
    a.chunks = v.chunk;
    a.header = v.header;
    a.films = v.films;
    a.wf = v.wf;
    a.counters = v.counters;
    a.refill_closest = refill_lanes(ctx->tuning.refill_closest);
    a.refill_any = refill_lanes(ctx->tuning.refill_any);
    const uint32_t n = uint32_t(npix);
    const uint32_t per = kNoAllocMaxPaths / n;  // samples per batch
    const int depth = sl.max_depth;
    ctx->batch_spheres = sl.has_spheres;
    ctx->stats = cgpu_render_stats{};
    for (uint32_t done = 0; done < num_samples;) {
        const uint32_t k = std::min(per, num_samples - done);
        BatchHeader h;
        h.num_chunks = 1;
        h.total_paths = k * n;
        h.total_pixels = n;
        h.max_depth = depth;
        h.seed = seed;
        const Chunk c{scene, 0, n, uint32_t(sl.width), first_sample + done, k, 0, 0};
        k_noalloc_setup<<<1, 256, 0, ctx->stream>>>(v, h, c, sl.d, sl.film, scene, (depth + 2) * kCntStride);
        enqueue_wavefront_serial(ctx, a, depth, k * n, n);
        ctx->stats.batches += 1;
        ctx->stats.paths += uint64_t(k) * n;
        done += k;
    }
    return cg_cuda(ctx, cudaGetLastError(), "render_noalloc launch");
}
