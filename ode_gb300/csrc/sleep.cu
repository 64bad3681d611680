// Auto-disable (sleeping) on the device: the per-body idle test of
// util.cpp:427-561 (dInternalHandleAutoDisabling), then the island rule of
// util.cpp:724-860 (BuildIslandsAndEstimateStepperMemoryRequirements) that
// decides which bodies a step processes:
//
//   * a body with auto-disable on, enabled, attached to at least one joint
//     (contact joints of this step included) and a non-zero sample count
//     records its velocities in a ring buffer of `average_samples` entries;
//     once the buffer is full, an average whose squared linear and angular
//     speeds are both within the thresholds counts as idle; idle steps count
//     down `idle_steps` and `idle_time`, a moving step resets them; when both
//     have run out the body is disabled and its velocities are zeroed;
//   * the reference walks the body-joint graph from every enabled body and
//     re-enables every body it reaches: so a connected component (bodies
//     joined by contacts and joints; the static environment joins nothing)
//     is processed, and all of its bodies enabled, when it holds at least one
//     enabled body; a component of disabled bodies only is not stepped at
//     all: no gravity, no rows, no integration, force accumulators kept.
//
// The components come from a lock-free union-find (hooking the larger root
// under the smaller with atomicCAS, path halving in find); every loop is
// bounded by the body count.  Contacts of sleeping components are removed by
// an order-preserving compaction into a second contact array (a manifold --
// consecutive contacts of one geom pair -- is kept or dropped as a whole),
// with the map back to the caller's contact index for joint feedback; joints
// of sleeping components get no rows (their row count is set to 0 by the
// joint getInfo1 kernel).
#include "gbode_internal.h"

namespace gb {

// --- per-body idle test (util.cpp:427-561)
__global__ void k_adis(Bodies B, int4 *ai, float4 *af, float4 *buf, int S, const int *touch, float h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    if (!touch[i]) return;  // not attached to any joint: never frozen mid-air
    int4 a = ai[i];
    if ((a.x & (GB_ADIS_ON | GB_ADIS_DISABLED)) != GB_ADIS_ON) return;
    const int samples = a.w;
    if (samples <= 0) return;
    int counter = (a.x >> 8) & 0xffff;
    int ready = (a.x & GB_ADIS_READY) != 0;
    if (counter >= samples) { ready = 0; counter = 0; }  // the reference's buffer sanity reset
    float4 lv = B.lvel[i], av = B.avel[i];
    float4 *rb = buf + (size_t)i * S * 2;
    rb[2 * counter] = lv;
    rb[2 * counter + 1] = av;
    counter++;
    if (counter >= samples) { counter = 0; ready = 1; }
    int idle = 0;
    if (ready) {
        idle = 1;
        float4 l0 = rb[0], a0 = rb[1];
        float al[3] = {l0.x, l0.y, l0.z}, aa[3] = {a0.x, a0.y, a0.z};
        if (samples > 1) {
            for (int k = 1; k < samples; k++) {
                const float4 l = rb[2 * k], w = rb[2 * k + 1];
                al[0] += l.x; aa[0] += w.x; al[1] += l.y; aa[1] += w.y; al[2] += l.z; aa[2] += w.z;
            }
            const float r1 = 1.0f / (float)samples;
            al[0] *= r1; aa[0] *= r1; al[1] *= r1; aa[1] *= r1; al[2] *= r1; aa[2] *= r1;
        }
        const float4 f = af[i];
        const float ls = al[0] * al[0] + al[1] * al[1] + al[2] * al[2];
        if (ls > f.x) idle = 0;
        else {
            const float as = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
            if (as > f.y) idle = 0;
        }
    }
    float4 f = af[i];
    if (idle) { a.z--; f.w -= h; }
    else { a.z = a.y; f.w = f.z; }
    int flags = (a.x & 0xff & ~GB_ADIS_READY) | (ready ? GB_ADIS_READY : 0) | (counter << 8);
    if (a.z <= 0 && f.w <= 0) {
        flags |= GB_ADIS_DISABLED;
        B.lvel[i] = make_float4(0.f, 0.f, 0.f, lv.w);  // .w: mass
        B.avel[i] = make_float4(0.f, 0.f, 0.f, av.w);  // .w: flag bits
    }
    a.x = flags;
    ai[i] = a;
    af[i] = f;
}

__global__ void k_sleep_touch(const Contact *C, const int *nc_dev, const int4 *jinfo, int nj, int *touch,
                              int *parent, int nb) {
    const int nc = *nc_dev;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int c = tid; c < nc; c += nth) {
        const Contact k = C[c];
        if (k.b1 >= 0) touch[k.b1] = 1;
        if (k.b2 >= 0) touch[k.b2] = 1;
    }
    for (int j = tid; j < nj; j += nth) {
        const int4 in = jinfo[j];
        if (in.y >= 0) touch[in.y] = 1;
        if (in.z >= 0) touch[in.z] = 1;
    }
    for (int i = tid; i < nb; i += nth) parent[i] = i;
}

// find with path halving; parents only ever point to smaller indices, so the
// walk ends within nb steps.  Loads go through L2 (__ldcg): another SM's hook
// must be seen, or a stale root would make the merge loop below spin.
__device__ __forceinline__ int uf_find(int *parent, int x) {
    int p = __ldcg(parent + x);
    while (p != x) {
        const int g = __ldcg(parent + p);
        if (g != p) parent[x] = g;  // benign race: any ancestor is a valid parent
        x = p;
        p = __ldcg(parent + x);
    }
    return x;
}

__device__ void uf_unite(int *parent, int a, int b, unsigned *err, int nb) {
    for (int guard = 0; guard <= nb; guard++) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
    atomicOr(err, ERR_ISLAND_LIMIT);
}

__global__ void k_sleep_link(const Contact *C, const int *nc_dev, const int4 *jinfo, int nj, int *parent,
                             unsigned *err, int nb) {
    const int nc = *nc_dev;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int c = tid; c < nc; c += nth) {
        const Contact k = C[c];
        if (k.b1 >= 0 && k.b2 >= 0 && k.b1 != k.b2) uf_unite(parent, k.b1, k.b2, err, nb);
    }
    for (int j = tid; j < nj; j += nth) {
        const int4 in = jinfo[j];
        if (in.y >= 0 && in.z >= 0 && in.y != in.z) uf_unite(parent, in.y, in.z, err, nb);
    }
}

__global__ void k_sleep_roots(int *parent, const int4 *ai, int *awake, int nb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int r = uf_find(parent, i);
    parent[i] = r;
    if (!(ai[i].x & GB_ADIS_DISABLED)) awake[r] = 1;
}

__global__ void k_sleep_apply(const int *parent, const int *awake, int4 *ai, int *asleep, DevCounters *dc, int nb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    if (awake[parent[i]]) {
        // reached from an enabled body: enabled again, countdowns untouched
        int4 a = ai[i];
        if (a.x & GB_ADIS_DISABLED) { a.x &= ~GB_ADIS_DISABLED; ai[i] = a; }
        asleep[i] = 0;
    } else {
        asleep[i] = 1;
        atomicAdd(&dc->nasleep, 1);
    }
}

__global__ void k_sleep_keep(const Contact *C, const int *nc_dev, const int *asleep, int *keep) {
    const int nc = *nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Contact k = C[c];
        const int b = k.b1 >= 0 ? k.b1 : k.b2;
        keep[c] = b >= 0 && !asleep[b];
    }
}

__global__ void k_sleep_scatter(const Contact *C, const int *nc_dev, const int *keep, const int *pos, Contact *out,
                                int *orig) {
    const int nc = *nc_dev;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (!keep[c]) continue;
        out[pos[c]] = C[c];
        orig[pos[c]] = c;
    }
}

bool ensure_sleep(Workspace &ws, int nb, int S) {
    const size_t n = nb > 0 ? nb : 1;
    const size_t s = S > 0 ? S : 1;
    return ws.b_adis_i.ensure(n * 16) && ws.b_adis_f.ensure(n * 16) && ws.b_adis_buf.ensure(n * s * 32) &&
           ws.b_touch.ensure(n * 4) && ws.b_parent.ensure(n * 4) && ws.b_awake.ensure(n * 4) &&
           ws.b_asleep.ensure(n * 4);
}

// The sleep stage of one step, before any body or row kernel: the idle test,
// the components, the asleep flags, and the compacted contact array the
// solver then reads (ws.c_awake, dc->nawake, ws.c_orig).
bool launch_sleep(Workspace &ws, int nb, float h, cudaStream_t s) {
    const size_t ncap = ws.contact_cap > 0 ? ws.contact_cap : 1;
    if (!(ws.c_keep.ensure(ncap * 4) && ws.c_kpos.ensure(ncap * 4) && ws.c_awake.ensure(ncap * sizeof(Contact)) &&
          ws.c_orig.ensure(ncap * 4)))
        return false;
    const Contact *C = ws.contacts.as<Contact>();
    const int grid = 4 * num_sms();
    const int nbg = nb > 0 ? (nb + 255) / 256 : 1;
    int *touch = ws.b_touch.as<int>(), *parent = ws.b_parent.as<int>(), *awake = ws.b_awake.as<int>();
    int *asleep = ws.b_asleep.as<int>();
    int4 *ai = ws.b_adis_i.as<int4>();
    cudaMemsetAsync(touch, 0, (size_t)(nb > 0 ? nb : 1) * 4, s);
    cudaMemsetAsync(awake, 0, (size_t)(nb > 0 ? nb : 1) * 4, s);
    cudaMemsetAsync(&ws.dc->nasleep, 0, 4, s);
    k_sleep_touch<<<grid, 256, 0, s>>>(C, &ws.dc->ncontacts, ws.j_info.as<int4>(), ws.njoints, touch, parent, nb);
    Bodies B = bodies_view(ws, nb);
    B.asleep = nullptr;
    k_adis<<<nbg, 256, 0, s>>>(B, ai, ws.b_adis_f.as<float4>(), ws.b_adis_buf.as<float4>(), ws.adis_S, touch, h);
    k_sleep_link<<<grid, 256, 0, s>>>(C, &ws.dc->ncontacts, ws.j_info.as<int4>(), ws.njoints, parent, &ws.dc->err, nb);
    k_sleep_roots<<<nbg, 256, 0, s>>>(parent, ai, awake, nb);
    k_sleep_apply<<<nbg, 256, 0, s>>>(parent, awake, ai, asleep, ws.dc, nb);
    k_sleep_keep<<<grid, 256, 0, s>>>(C, &ws.dc->ncontacts, asleep, ws.c_keep.as<int>());
    scan_exclusive(ws.c_keep.as<int>(), ws.c_kpos.as<int>(), &ws.dc->ncontacts, ws.contact_cap, &ws.dc->nawake, ws, s);
    k_sleep_scatter<<<grid, 256, 0, s>>>(C, &ws.dc->ncontacts, ws.c_keep.as<int>(), ws.c_kpos.as<int>(),
                                         ws.c_awake.as<Contact>(), ws.c_orig.as<int>());
    count_launch(7);
    return cudaGetLastError() == cudaSuccess;
}

}  // namespace gb
