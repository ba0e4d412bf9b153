// pt_kernels.cu -- wavefront path tracing: ray generation, shading with
// next-event estimation, queue compaction and the per-pixel resolve.
// Compiled with --fmad=false (exact binary32 operation order, see snk_device.cuh).
//
// The reference's pass 2 shades every pixel in one ray-generation thread and
// adds a biased diffuse bounce (BounceDiffuse, Core/res/shaders/RayGen.rgen:139-213:
// cos(dot(...)) weight, x0.25 inner bounces).  This path tracer replaces it with an
// unbiased estimator for the reference's own BRDF (LightBuffers.glsl:104-144):
//   - emission counted on camera hits only; every vertex does NEE toward the
//     directional light (as RayClosestHit.rchit:136) and one power-sampled local
//     light (sphere light or emissive triangle);
//   - continuation samples a GGX-NDF / cosine mixture; its weight is
//     albedo * CookTorranceBRDF(l) / pdf for the reference's BRDF with albedo
//     applied to both terms (RayGen.rgen:273);
//   - russian roulette from segment rr_depth with survival min(max(beta), 0.95).
// Random numbers: PCG32 streams keyed by (pixel, sample, segment, seed); each
// vertex draws 7 numbers, the camera segment 2 more for the pixel jitter.
//
// In the ReSTIR + indirect mode (F.indirect) the same paths carry only the
// indirect light of the reference's pass 2 (RayGen.rgen:565-566): the primary
// vertex adds no emission and does no NEE (the ReSTIR passes shade it), its
// continuation starts the path, and every later vertex is shaded as above.  The
// first shading pass also writes the ReSTIR surface records of sample 0, whose
// camera ray goes through the pixel centre as the ReSTIR G-buffer's does.
#include "snk_frame.h"

namespace snk {
namespace {

constexpr int BLK = 256;

// Path p -> (global pixel, sample key, view, x, y).  In radiance-cache mode the
// paths from n_render on are training paths: pixel chosen by a hash of (path,
// frame), sample key 0x40000000 | index (its own random streams, jittered ray,
// no G-buffer writes).
__device__ __forceinline__ bool decode_path(const FrameParams& F, uint32_t p, uint32_t* gpix, uint32_t* s,
                                            uint32_t* vi, uint32_t* x, uint32_t* y) {
    bool train = F.cache && p >= F.n_render;
    if (!train) {
        *gpix = p / F.spp;
        *s = p - *gpix * F.spp;
    } else {
        const uint32_t tid = p - F.n_render;
        *gpix = (uint32_t)(splitmix64(((uint64_t)frame_index(F) << 32) | tid) % (uint64_t)F.n_pixels);
        *s = 0x40000000u | tid;
    }
    *vi = find_view(F.views, F.nviews, *gpix);
    const ViewDev& V = F.views[*vi];
    uint32_t local = *gpix - V.pixel_offset;
    *x = local % V.v.width;
    *y = local / V.v.width;
    return train;
}

// Path of camera-ray queue entry q: for warp packets (F.packet_primary) the pixels
// of each view are queued in PACKET_TILE_W x PACKET_TILE_H tiles (row-major tiles,
// row-major pixels within a tile), so a warp's 32 rays cover a compact patch of the
// image; otherwise, and for the training paths of the radiance cache, in path order.
__device__ __forceinline__ uint32_t queue_path(const FrameParams& F, uint32_t q) {
    if (!F.packet_primary || (F.cache && q >= F.n_render)) return q;
    const uint32_t g = q / F.spp, s = q - g * F.spp;
    const ViewDev& V = F.views[find_view(F.views, F.nviews, g)];
    const uint32_t r = g - V.pixel_offset, t = r >> 5, w = r & 31u, tiles_x = V.v.width / PACKET_TILE_W;
    const uint32_t x = (t % tiles_x) * PACKET_TILE_W + w % PACKET_TILE_W,
                   y = (t / tiles_x) * PACKET_TILE_H + w / PACKET_TILE_W;
    return (V.pixel_offset + y * V.v.width + x) * F.spp + s;
}

__global__ void __launch_bounds__(BLK) k_generate(FrameParams F) {
    if (blockIdx.x == 0 && threadIdx.x == 0) F.counters[CNT_QUEUE + 0] = F.n_paths;
    for (uint32_t q = blockIdx.x * BLK + threadIdx.x; q < F.n_paths; q += gridDim.x * BLK) {
        const uint32_t p = queue_path(F, q);
        uint32_t gpix, s, vi, x, y;
        decode_path(F, p, &gpix, &s, &vi, &x, &y);
        const ViewDev& V = F.views[vi];
        Pcg rng = pcg_stream(gpix, s, 0u, frame_seed(F));
        float j1 = pcg_float(rng), j2 = pcg_float(rng);
        float jx = s == 0 ? 0.5f : j1, jy = s == 0 ? 0.5f : j2;
        V3 d = camera_dir(V.v, x, y, jx, jy);
        F.rays[0][2ull * q] = make_float4(V.v.pos[0], V.v.pos[1], V.v.pos[2], 0.0f);
        F.rays[0][2ull * q + 1] = make_float4(d.x, d.y, d.z, T_FAR);
        F.path_ids[0][q] = p;
        F.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        F.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (F.cache) F.spread[p] = make_float2(0.0f, 0.0f);
    }
}

__device__ __forceinline__ void write_gbuffer_hit(const ViewDev& V, uint32_t o, const Surface& s, float t, float2 mo) {
    if (V.albedo) V.albedo[o] = make_float4(s.albedo.x, s.albedo.y, s.albedo.z, 1.0f);
    if (V.normal) V.normal[o] = make_float4(s.n.x, s.n.y, s.n.z, 0.0f);
    if (V.position) V.position[o] = make_float4(s.pos.x, s.pos.y, s.pos.z, 1.0f);
    if (V.rma) V.rma[o] = make_float4(s.roughness, s.metallic, s.ao, 1.0f);
    if (V.motion) V.motion[o] = mo;
    if (V.depth) V.depth[o] = t;
    if (V.mat_flags) V.mat_flags[o] = s.flags;
    if (V.inst_id) V.inst_id[o] = s.inst;
    if (V.prim_id) V.prim_id[o] = s.prim;
}

__device__ __forceinline__ void write_gbuffer_miss(const ViewDev& V, uint32_t o) {
    float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (V.albedo) V.albedo[o] = z;
    if (V.normal) V.normal[o] = z;
    if (V.position) V.position[o] = z;
    if (V.rma) V.rma[o] = z;
    if (V.motion) V.motion[o] = make_float2(0.0f, 0.0f);
    if (V.depth) V.depth[o] = -1.0f;
    if (V.mat_flags) V.mat_flags[o] = 0u;
    if (V.inst_id) V.inst_id[o] = INVALID;
    if (V.prim_id) V.prim_id[o] = INVALID;
}

// 4 resident blocks per SM (64 registers): the kernel is bound by the latency of
// its dependent loads (path id -> hit -> triangle -> material), and twice the
// resident warps of the unconstrained 93-register build outweigh a few spills.
// Misses end in a first pass over each chunk of 32 queue entries (their shadow
// slots are marked empty and, on the first segment, the G-buffer gets a miss);
// hits are collected in a per-warp ring in shared memory and shaded 32 at a
// time, so the surface shading runs with full warps even when most rays of a
// bounce leave the scene.  Every output is indexed by queue entry or path, so
// the order in which entries are shaded does not change any result.
template <bool CACHE, bool FIRST>   // the MLP cache is on; FIRST (camera rays: G-buffer, emission)
__global__ void __launch_bounds__(BLK, 4) k_shade(FrameParams F, uint32_t d) {
    __shared__ uint32_t ring[BLK / 32][64];
    const uint32_t cur = d & 1u, nxt = cur ^ 1u;
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp_global = (blockIdx.x * BLK + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * BLK) >> 5;
    const SceneDev& S = F.S;
    uint32_t* hq = ring[threadIdx.x >> 5];
    uint32_t head = 0, cnt = 0;   // hits waiting in the ring (at most 63)
    for (uint32_t base = warp_global * 32u;; base += nwarps * 32u) {
        const bool more = base < n;
        if (more) {
            const uint32_t i = base + lane;
            bool hit = false;
            if (i < n) {
                hit = F.hits[i].flags != 0u;
                if (!hit) {   // no shadow rays: zero contributions
                    F.shadow_contrib[shadow_entry(F, i, 0)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    F.shadow_contrib[shadow_entry(F, i, 1)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (FIRST) {
                        uint32_t gpix, s, vi, x, y;
                        const bool train = decode_path(F, F.path_ids[cur][i], &gpix, &s, &vi, &x, &y);
                        if (s == 0 && !train) {
                            const ViewDev& V = F.views[vi];
                            write_gbuffer_miss(V, y * V.v.width + x);
                            if (V.rs_pos) write_restir_miss(V, y * V.v.width + x);
                        }
                    }
                    // the path ends here (after the G-buffer above has decoded its id)
                    if (F.early_resolve) F.path_ids[cur][i] |= 0x80000000u;
                }
            }
            const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
            if (hit) hq[(head + cnt + (uint32_t)__popc(hm & ((1u << lane) - 1u))) & 63u] = i;
            cnt += (uint32_t)__popc(hm);
            __syncwarp();
        }
        while (cnt >= 32u || (!more && cnt > 0u)) {
            const uint32_t take = cnt < 32u ? cnt : 32u;
            const bool have = lane < take;
            const uint32_t i = have ? hq[(head + lane) & 63u] : 0u;
            head = (head + take) & 63u;
            cnt -= take;
            __syncwarp();
            bool cont = false, sv0 = false, sv1 = false, query = false;
            uint32_t p = 0;
            float4 nr0 = make_float4(0, 0, 0, 0), nr1 = make_float4(0, 0, 0, 0);
            // shadow rays: their origin and the local-light ray's direction + tmax (the
            // directional-light ray's direction is the light's); contributions are
            // written where the rays are made
            float4 so = make_float4(0, 0, 0, 0), sd1 = so;
            float4 q0, q1, q2, q3, qb;
            if (have) {
                p = F.path_ids[cur][i];
                uint32_t gpix, s, vi, x, y;
                const bool train = decode_path(F, p, &gpix, &s, &vi, &x, &y);
                const ViewDev& V = F.views[vi];
                const uint32_t o = y * V.v.width + x;
                float4 rd4 = F.rays[cur][2ull * i + 1];
                V3 rd = v3(rd4.x, rd4.y, rd4.z);
                HitDev h = F.hits[i];
                Pcg rng = pcg_stream(gpix, s, d, frame_seed(F));
                if (FIRST) { pcg_next(rng); pcg_next(rng); }
                const bool gbuf = FIRST && s == 0 && !train;
                {   // a hit (misses ended in the first pass)
                    Surface sf = surface_at(S, h.inst, h.prim, h.u, h.v, rd);
                    if (gbuf) {
                        const float2 mo = motion_of(S, V.v, sf, x, y);
                        write_gbuffer_hit(V, o, sf, h.t, mo);
                        if (V.rs_pos) write_restir_surface(V, o, sf, mo);
                    }
                    // indirect mode: ReSTIR DI shades the primary vertex (no emission, no NEE here)
                    const bool direct = !(F.indirect && FIRST);
                    float u_sel = pcg_float(rng), u1 = pcg_float(rng), u2 = pcg_float(rng);
                    float u_rr = pcg_float(rng), u_d1 = pcg_float(rng), u_d2 = pcg_float(rng);
                    float u_lobe = pcg_float(rng);
                    float4 b4 = F.beta[p];
                    V3 beta = v3(b4.x, b4.y, b4.z);
                    bool to_cache = false;
                    if (CACHE) {
                        // path spread (Mueller et al. 2021): a0 = t^2 / (4 pi cos) at the primary
                        // vertex; later vertices add sqrt(t^2 / (pdf cos)); the path is handed
                        // to the cache once spread^2 > c a0
                        float2 sp = F.spread[p];
                        const float cosv = fmax_(fabsf(dot(sf.n, rd)), 1e-6f);
                        if (FIRST) sp = make_float2((h.t * h.t) / ((4.0f * PI) * cosv), 0.0f);
                        else sp.y = sp.y + sqrtf((h.t * h.t) / (fmax_(b4.w, 1e-6f) * cosv));
                        F.spread[p] = sp;
                        to_cache = !train && !FIRST && !(sf.flags & MAT_EMISSIVE) && (sp.y * sp.y > F.spread_c * sp.x);
                        if (train && d < TRAIN_V && !(sf.flags & MAT_EMISSIVE)) {
                            const uint32_t slot = (p - F.n_render) * TRAIN_V + d;
                            float4* r = F.train_rec + 4ull * slot;
                            r[0] = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, sf.roughness);
                            r[1] = make_float4(-rd.x, -rd.y, -rd.z, sf.metallic);
                            r[2] = make_float4(sf.n.x, sf.n.y, sf.n.z, 0.0f);
                            r[3] = make_float4(sf.albedo.x, sf.albedo.y, sf.albedo.z, 0.0f);
                            F.train_beta[slot] = make_float4(beta.x, beta.y, beta.z, 1.0f);
                        }
                    }
                    if (to_cache) {
                        q0 = make_float4(sf.pos.x, sf.pos.y, sf.pos.z, sf.roughness);
                        q1 = make_float4(-rd.x, -rd.y, -rd.z, sf.metallic);
                        q2 = make_float4(sf.n.x, sf.n.y, sf.n.z, 0.0f);
                        q3 = make_float4(sf.albedo.x, sf.albedo.y, sf.albedo.z, __uint_as_float(p));
                        qb = make_float4(beta.x, beta.y, beta.z, 0.0f);
                        query = true;
                    } else if (sf.flags & MAT_EMISSIVE) {
                        if (FIRST && direct) {
                            float4 l4 = F.L[p];
                            V3 Lp = add(v3(l4.x, l4.y, l4.z), cmul(beta, sf.albedo));
                            F.L[p] = make_float4(Lp.x, Lp.y, Lp.z, 0.0f);
                        }
                    } else {
                        V3 v = neg(rd);
                        V3 f0 = f0_of(sf.albedo, sf.metallic);
                        V3 xb = add(sf.pos, mul(sf.n, SURFACE_BIAS));
                        if (direct && S.dir_light.enabled) {
                            V3 c = calc_directional(load3(S.dir_light.dir), load3(S.dir_light.colour), v, f0, sf.n,
                                                    sf.roughness, sf.metallic, sf.albedo);
                            if (maxc(c) > 0.0f) {
                                V3 cb = cmul(beta, c);
                                F.shadow_contrib[shadow_entry(F, i, 0)] = make_float4(cb.x, cb.y, cb.z, 0.0f);
                                sv0 = true;
                            }
                        }
                        V3 c, ldir;
                        float ltmax;
                        if (direct && sample_local(S, sf, v, f0, xb, u_sel, u1, u2, &c, &ldir, &ltmax)) {
                            V3 cb = cmul(beta, c);
                            sd1 = make_float4(ldir.x, ldir.y, ldir.z, ltmax);
                            F.shadow_contrib[shadow_entry(F, i, 1)] = make_float4(cb.x, cb.y, cb.z, 0.0f);
                            sv1 = true;
                        }
                        so = make_float4(xb.x, xb.y, xb.z, 0.0f);
                        bool alive = d + 1 < F.max_depth;
                        if (alive && d + 1 >= F.rr_depth) {
                            float ps = fmin_(maxc(beta), 0.95f);
                            if (u_rr < ps) beta = v3(beta.x / ps, beta.y / ps, beta.z / ps);
                            else alive = false;
                        }
                        if (alive) {
                            V3 wi, w;
                            float pdf;
                            if (sample_continuation(sf, v, f0, u_lobe, u_d1, u_d2, &wi, &w, &pdf)) {
                                beta = cmul(beta, w);
                                // w: pdf of the sampled direction, used by the spread heuristic
                                F.beta[p] = make_float4(beta.x, beta.y, beta.z, pdf);
                                nr0 = make_float4(xb.x, xb.y, xb.z, EXT_TMIN);
                                nr1 = make_float4(wi.x, wi.y, wi.z, T_FAR);
                                cont = true;
                            }
                        }
                    }
                }
            }
            if (have) {   // zero contribution: no shadow ray of that kind
                const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (!sv0) F.shadow_contrib[shadow_entry(F, i, 0)] = z;
                if (!sv1) F.shadow_contrib[shadow_entry(F, i, 1)] = z;
            }
            // warp-ballot compaction of the continuing paths into the next queue and of
            // the shadow rays into their kinds' parts of the shadow queue
            const unsigned full = 0xFFFFFFFFu;
            const unsigned m = __ballot_sync(full, cont);
            const unsigned m0 = __ballot_sync(full, sv0), m1 = __ballot_sync(full, sv1);
            const unsigned lt = (1u << lane) - 1u;
            uint32_t slot_base = 0, b0 = 0, b1 = 0;
            if (lane == 0) {
                if (m) slot_base = atomicAdd(&F.counters[CNT_QUEUE + d + 1], (uint32_t)__popc(m));
                if (m0) b0 = atomicAdd(&F.counters[CNT_SHADOW_Q + 2 * d], (uint32_t)__popc(m0));
                if (m1) b1 = atomicAdd(&F.counters[CNT_SHADOW_Q + 2 * d + 1], (uint32_t)__popc(m1));
                if (m0 | m1) atomicAdd(&F.counters[CNT_SHADOW_RAYS], (uint32_t)(__popc(m0) + __popc(m1)));
            }
            slot_base = __shfl_sync(full, slot_base, 0);
            b0 = __shfl_sync(full, b0, 0);
            b1 = __shfl_sync(full, b1, 0);
            if (cont) {
                uint32_t j = slot_base + __popc(m & lt);
                F.rays[nxt][2ull * j] = nr0;
                F.rays[nxt][2ull * j + 1] = nr1;
                F.path_ids[nxt][j] = p;
            } else if (have && F.early_resolve) {
                F.path_ids[cur][i] = p | 0x80000000u;   // the path ends in this segment
            }
            if (sv0) {   // (the origin's w carries the bits of the contribution entry)
                const size_t e = b0 + (uint32_t)__popc(m0 & lt);
                F.shadow_rays[2 * e] = make_float4(so.x, so.y, so.z, __uint_as_float((uint32_t)shadow_entry(F, i, 0)));
                F.shadow_rays[2 * e + 1] = make_float4(S.dir_light.dir[0], S.dir_light.dir[1], S.dir_light.dir[2], T_FAR);
            }
            if (sv1) {
                const size_t e = (size_t)F.n_paths + b1 + (uint32_t)__popc(m1 & lt);
                F.shadow_rays[2 * e] = make_float4(so.x, so.y, so.z, __uint_as_float((uint32_t)shadow_entry(F, i, 1)));
                F.shadow_rays[2 * e + 1] = sd1;
            }
            if (CACHE) {
                const unsigned qm = __ballot_sync(full, query);
                uint32_t qbase = 0;
                if (lane == 0 && qm) qbase = atomicAdd(&F.counters[CNT_CACHE_QUERIES], (uint32_t)__popc(qm));
                qbase = __shfl_sync(full, qbase, 0);
                if (query) {
                    const uint32_t j = qbase + __popc(qm & ((1u << lane) - 1u));
                    F.qrec[4ull * j] = q0;
                    F.qrec[4ull * j + 1] = q1;
                    F.qrec[4ull * j + 2] = q2;
                    F.qrec[4ull * j + 3] = q3;
                    F.qbeta[j] = qb;
                }
            }
        }
        if (!more) break;
    }
}

// training samples of the cache: target at recorded vertex i of a training path =
// (radiance gathered at vertices i, i+1, ...) / throughput at i; weight 0 when the
// vertex was not reached or its throughput has a zero channel
__global__ void __launch_bounds__(BLK) k_make_samples(FrameParams F) {
    const uint32_t n = F.n_train * TRAIN_V;
    for (uint32_t idx = blockIdx.x * BLK + threadIdx.x; idx < n; idx += gridDim.x * BLK) {
        const uint32_t tid = idx / TRAIN_V, i = idx - tid * TRAIN_V;
        const float4 b = F.train_beta[idx];
        const bool valid = b.w != 0.0f && b.x > 0.0f && b.y > 0.0f && b.z > 0.0f;
        float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t k = i; k < TRAIN_V; k++) {
            const float4 l = F.train_L[tid * TRAIN_V + k];
            sum = make_float4(sum.x + l.x, sum.y + l.y, sum.z + l.z, 0.0f);
        }
        float4* s = F.samples + 5ull * idx;
        const float4* r = F.train_rec + 4ull * idx;
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        s[0] = valid ? r[0] : z;
        s[1] = valid ? r[1] : z;
        s[2] = valid ? r[2] : z;
        s[3] = valid ? r[3] : z;
        s[4] = valid ? make_float4(sum.x / b.x, sum.y / b.y, sum.z / b.z, 1.0f) : z;
    }
}

__global__ void __launch_bounds__(BLK) k_resolve(FrameParams F) {
    const float inv = 1.0f / (float)F.spp;
    for (uint32_t g = blockIdx.x * BLK + threadIdx.x; g < F.n_pixels; g += gridDim.x * BLK) {
        uint32_t vi = find_view(F.views, F.nviews, g);
        const ViewDev& V = F.views[vi];
        uint32_t o = g - V.pixel_offset;
        V3 sum = v3(0.0f, 0.0f, 0.0f);
        for (uint32_t s = 0; s < F.spp; s++) {
            float4 l = F.L[(size_t)g * F.spp + s];
            sum = add(sum, v3(l.x, l.y, l.z));
        }
        float4 r = make_float4(sum.x * inv, sum.y * inv, sum.z * inv, 1.0f);
        if (F.indirect) {   // the ReSTIR final pass adds it to the pixel's direct light
            F.indirect_out[g] = r;
            continue;
        }
        if (V.radiance) V.radiance[o] = r;
        if (vi == 0 && frame_accumulate(F)) {
            double2 a0 = F.accum[2ull * o], a1 = F.accum[2ull * o + 1];
            a0.x += (double)r.x; a0.y += (double)r.y; a1.x += (double)r.z; a1.y += 1.0;
            F.accum[2ull * o] = a0;
            F.accum[2ull * o + 1] = a1;
        }
    }
}

}  // namespace

cudaError_t launch_generate(const FrameParams& F, int grid, cudaStream_t s) {
    k_generate<<<grid, BLK, 0, s>>>(F);
    return cudaGetLastError();
}
cudaError_t launch_shade(const FrameParams& F, uint32_t depth, int grid, cudaStream_t s) {
    const bool cache = F.cache != 0, first = depth == 0;
    if (cache) {
        if (first) k_shade<true, true><<<grid, BLK, 0, s>>>(F, depth);
        else k_shade<true, false><<<grid, BLK, 0, s>>>(F, depth);
    } else {
        if (first) k_shade<false, true><<<grid, BLK, 0, s>>>(F, depth);
        else k_shade<false, false><<<grid, BLK, 0, s>>>(F, depth);
    }
    return cudaGetLastError();
}
cudaError_t launch_resolve(const FrameParams& F, int grid, cudaStream_t s) {
    k_resolve<<<grid, BLK, 0, s>>>(F);
    return cudaGetLastError();
}
cudaError_t launch_make_samples(const FrameParams& F, int grid, cudaStream_t s) {
    k_make_samples<<<grid, BLK, 0, s>>>(F);
    return cudaGetLastError();
}

}  // namespace snk
