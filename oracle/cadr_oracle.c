/*
 * cadr_oracle.c - CPU oracle of the drawable-processing pass.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA path is compared against and
 * the timed CPU baseline.  See cadr_oracle.h for what each function restates.  Must be
 * compiled with -ffp-contract=off (oracle/Makefile does).
 */
#include "cadr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void set_threads(int threads)
{
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

/* ---------------------------------------------------------------------- */
/* Tier A: processDrawables.comp:77-113. */

typedef struct image_view {
    const oracle_region* r;
    uint32_t n;
    int bad;
} image_view;

/* Host bytes of [addr, addr + len) when one region holds all of them. */
static const uint8_t* locate(image_view* im, uint64_t addr, uint64_t len)
{
    for (uint32_t k = 0; k < im->n; k++) {
        const oracle_region* g = &im->r[k];
        if (g->size >= len && addr >= g->base && addr - g->base <= g->size - len)
            return g->bytes + (addr - g->base);
    }
    im->bad = 1;
    return NULL;
}

static uint64_t rd64(image_view* im, uint64_t addr)
{
    const uint8_t* p = locate(im, addr, 8);
    uint64_t v = 0;
    if (p) memcpy(&v, p, 8);
    return v;
}

static uint32_t rd32(image_view* im, uint64_t addr)
{
    const uint8_t* p = locate(im, addr, 4);
    uint32_t v = 0;
    if (p) memcpy(&v, p, 4);
    return v;
}

/* lookupHandle, processDrawables.comp:77-89.  Each index is the 32-bit
 * truncation the shader applies with uint(...). */
static uint64_t lookup_handle(image_view* im, uint32_t level, uint64_t root, uint64_t h)
{
    if (level == 1) return rd64(im, root + 8ull * (uint32_t)h);
    if (level == 2) {
        uint64_t t2 = rd64(im, root + 8ull * (uint32_t)(h >> 11));
        return rd64(im, t2 + 8ull * ((uint32_t)h & 0x7ffu));
    }
    uint64_t t2 = rd64(im, root + 8ull * (uint32_t)(h >> 22));
    uint64_t t3 = rd64(im, t2 + 8ull * ((uint32_t)(h >> 11) & 0x7ffu));
    return rd64(im, t3 + 8ull * ((uint32_t)h & 0x7ffu));
}

int oracle_process_drawables(const uint8_t* image, uint64_t image_base, uint64_t image_size,
                             uint32_t handle_level, uint64_t handle_table_addr,
                             const cadr_drawable_gpu_data* drawables, uint64_t n,
                             cadr_draw_indirect_cmd* indirect, cadr_drawable_pointers* pointers,
                             int threads)
{
    const oracle_region r = {image, image_base, image_size};
    return oracle_process_drawables_regions(&r, 1, handle_level, handle_table_addr, drawables, n,
                                            indirect, pointers, threads);
}

int oracle_process_drawables_regions(const oracle_region* regions, uint32_t num_regions,
                                     uint32_t handle_level, uint64_t handle_table_addr,
                                     const cadr_drawable_gpu_data* drawables, uint64_t n,
                                     cadr_draw_indirect_cmd* indirect,
                                     cadr_drawable_pointers* pointers, int threads)
{
    if (handle_level < 1 || handle_level > 3) return -1;
    int bad = 0;
    set_threads(threads);
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        image_view im = {regions, num_regions, 0};
        const cadr_drawable_gpu_data* d = &drawables[i];
        /* main(), processDrawables.comp:95-112 */
        uint64_t ps = lookup_handle(&im, handle_level, handle_table_addr, d->primitive_set_handle) +
                      (uint64_t)d->primitive_set_offset;
        uint64_t ml = lookup_handle(&im, handle_level, handle_table_addr, d->matrix_list_handle);
        indirect[i].vertex_count = rd32(&im, ps);
        indirect[i].instance_count = rd32(&im, ml);
        indirect[i].first_vertex = rd32(&im, ps + 4);
        indirect[i].first_instance = 0;
        pointers[i].vertex_data_ptr =
            lookup_handle(&im, handle_level, handle_table_addr, d->vertex_data_handle);
        pointers[i].index_data_ptr =
            lookup_handle(&im, handle_level, handle_table_addr, d->index_data_handle);
        pointers[i].matrix_list_ptr = ml;
        pointers[i].drawable_data_ptr =
            lookup_handle(&im, handle_level, handle_table_addr, d->drawable_data_handle);
        bad |= im.bad;
    }
    return bad ? -1 : 0;
}

/* ---------------------------------------------------------------------- */
/* Tier B arithmetic. */

/* GLM mat4 * mat4 (glm/detail/type_mat4x4.inl operator*):
 *   Result[c] = SrcA0*B[c][0] + SrcA1*B[c][1] + SrcA2*B[c][2] + SrcA3*B[c][3]
 * evaluated left to right, one rounding per operation. */
void oracle_mat4_mul(const float* a, const float* b, float* out)
{
    float r[16];
    for (int c = 0; c < 4; c++) {
        const float b0 = b[c * 4 + 0], b1 = b[c * 4 + 1], b2 = b[c * 4 + 2], b3 = b[c * 4 + 3];
        for (int k = 0; k < 4; k++) {
            float t = a[0 * 4 + k] * b0;
            t = t + a[1 * 4 + k] * b1;
            t = t + a[2 * 4 + k] * b2;
            t = t + a[3 * 4 + k] * b3;
            r[c * 4 + k] = t;
        }
    }
    memcpy(out, r, sizeof(r));
}

/* BoundingSphere operator*, src/CadR/BoundingSphere.h:70-86:
 *   center = mat3(M) * c + vec3(M[3])   (GLM mat3*vec3: m[0][k]*x + m[1][k]*y + m[2][k]*z)
 *   radius = sqrt(max(max(len2(M[0]), len2(M[1])), len2(M[2]))) * r
 * with len2(x,y,z) = x*x + y*y + z*z, std::max(a,b) = (a < b) ? b : a, and
 * the square root and the product by r evaluated in double. */
void oracle_sphere_transform(const float* m, const float* s, float* out)
{
    float c[3];
    for (int k = 0; k < 3; k++) {
        float t = m[0 * 4 + k] * s[0];
        t = t + m[1 * 4 + k] * s[1];
        t = t + m[2 * 4 + k] * s[2];
        c[k] = t + m[3 * 4 + k];
    }
    float l[3];
    for (int col = 0; col < 3; col++) {
        const float x = m[col * 4 + 0], y = m[col * 4 + 1], z = m[col * 4 + 2];
        float t = x * x;
        t = t + y * y;
        l[col] = t + z * z;
    }
    float mx = (l[0] < l[1]) ? l[1] : l[0];
    mx = (mx < l[2]) ? l[2] : mx;
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
    /* BoundingSphere.h:85 calls unqualified sqrt() on a float inside
     * namespace CadR, which resolves to the C library's double sqrt(double):
     * the reference computes the radius in double and rounds it once to
     * float on return. */
    out[3] = (float)(sqrt((double)mx) * (double)s[3]);
}

int oracle_propagate(const float* parent_world, uint64_t num_parents, const float* local,
                     const uint32_t* parent, uint64_t n, float* world, int threads)
{
    int bad = 0;
    set_threads(threads);
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        if (!parent) {
            memcpy(world + 16 * i, local + 16 * i, 64);
            continue;
        }
        uint32_t p = parent[i];
        if (p >= num_parents) {
            bad = 1;
            continue;
        }
        oracle_mat4_mul(parent_world + 16ull * p, local + 16 * i, world + 16 * i);
    }
    return bad ? -1 : 0;
}

/* Plane test, marginal band and LOD of one world sphere (project spec):
 *   dist_p  = ((nx*cx + ny*cy) + nz*cz) + d
 *   visible = dist_p >= -r for all six planes
 *   marginal= |dist_p + r| <= 1e-5 for some plane: the sphere's surface lies
 *             within 1e-5 of that plane (an absolute band, in world units)
 *   zc      = perspective ? max(-z_view, near) : 1, z_view = ((vz0*cx+vz1*cy)+vz2*cz)+vz3
 *   lod     = first k < L-1 with r*lod_scale >= T[k]*zc, else L-1 */
void oracle_classify(const float* ws, const cadr_view* v, uint32_t num_lods, int* visible,
                     uint32_t* lod, int* marginal)
{
    const float cx = ws[0], cy = ws[1], cz = ws[2], r = ws[3];
    int vis = 1, mar = 0;
    for (int p = 0; p < 6; p++) {
        const float* pl = v->planes[p];
        float dist = pl[0] * cx;
        dist = dist + pl[1] * cy;
        dist = dist + pl[2] * cz;
        dist = dist + pl[3];
        if (!(dist >= -r)) vis = 0;
        float t = dist + r;
        if (fabsf(t) <= 1e-5f) mar = 1;
    }
    float zc = 1.0f;
    if (v->perspective) {
        float z = v->view_z[0] * cx;
        z = z + v->view_z[1] * cy;
        z = z + v->view_z[2] * cz;
        z = z + v->view_z[3];
        zc = fmaxf(-z, v->near_z);
    }
    const float s = r * v->lod_scale;
    uint32_t l = num_lods - 1;
    for (uint32_t k = 0; k + 1 < num_lods; k++) {
        if (s >= v->lod_threshold[k] * zc) {
            l = k;
            break;
        }
    }
    *visible = vis;
    *lod = l;
    *marginal = mar;
}

static int check_offsets(uint64_t n, uint32_t S, const uint32_t* off)
{
    if (S == 0 || off[0] != 0 || off[S] != n) return -1;
    for (uint32_t s = 0; s < S; s++)
        if (off[s + 1] < off[s]) return -1;
    return 0;
}

/* Per-StateSet compaction: visible drawables of StateSet s, in ascending
 * drawable order, fill cmds[off[s] ...]; counts[s] is their number.  The
 * regions are the reference's contiguous StateSet regions
 * (src/CadR/StateSet.cpp:233-261). */
static int compact(uint64_t n, const uint8_t* vis, const uint8_t* lodv, const uint32_t* geometry,
                   uint32_t S, const uint32_t* off, uint32_t G, uint32_t L, const cadr_lod* lods,
                   cadr_draw_indexed_cmd* cmds, uint32_t* counts)
{
    (void)n;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
    for (int64_t s = 0; s < (int64_t)S; s++) {
        uint32_t k = 0;
        for (uint32_t i = off[s]; i < off[s + 1]; i++) {
            if (!vis[i]) continue;
            uint32_t g = geometry[i];
            if (g >= G) {
                bad = 1;
                continue;
            }
            const cadr_lod* e = &lods[(uint64_t)g * L + lodv[i]];
            cadr_draw_indexed_cmd* c = &cmds[off[s] + k];
            c->index_count = e->index_count;
            c->instance_count = 1;
            c->first_index = e->first_index;
            c->vertex_offset = e->vertex_offset;
            c->first_instance = i;
            k++;
        }
        counts[s] = k;
    }
    return bad ? -1 : 0;
}

static void classify_all(uint64_t n, const float* ws, const cadr_view* view, uint32_t L,
                         uint8_t* vis, uint8_t* lodv, uint32_t* marginal)
{
    if (marginal) memset(marginal, 0, ((n + 31) / 32) * 4);
#pragma omp parallel for schedule(static)
    for (int64_t w = 0; w < (int64_t)((n + 31) / 32); w++) {
        uint32_t bits = 0;
        for (uint64_t i = (uint64_t)w * 32; i < n && i < (uint64_t)w * 32 + 32; i++) {
            int v, m;
            uint32_t l;
            oracle_classify(ws + 4 * i, view, L, &v, &l, &m);
            vis[i] = (uint8_t)v;
            lodv[i] = (uint8_t)l;
            if (m) bits |= 1u << (i & 31);
        }
        if (marginal) marginal[w] = bits;
    }
}

int oracle_cull_spheres(uint64_t n, const float* world_sphere, const uint32_t* geometry,
                        uint32_t S, const uint32_t* off, uint32_t G, uint32_t L,
                        const cadr_lod* lods, const cadr_view* view, cadr_draw_indexed_cmd* cmds,
                        uint32_t* counts, uint32_t* marginal, int threads)
{
    if (L < 1 || L > 4 || check_offsets(n, S, off)) return -1;
    set_threads(threads);
    uint8_t* vis = (uint8_t*)malloc(n ? n : 1);
    uint8_t* lodv = (uint8_t*)malloc(n ? n : 1);
    if (!vis || !lodv) {
        free(vis);
        free(lodv);
        return -1;
    }
    classify_all(n, world_sphere, view, L, vis, lodv, marginal);
    int rc = compact(n, vis, lodv, geometry, S, off, G, L, lods, cmds, counts);
    free(vis);
    free(lodv);
    return rc;
}

int oracle_cull(uint32_t num_levels, const uint64_t* level_size, const float* const* level_local,
                const uint32_t* const* level_parent, uint64_t n, const float* local,
                const uint32_t* parent, const float* sphere, const uint32_t* geometry, uint32_t S,
                const uint32_t* off, uint32_t G, uint32_t L, const cadr_lod* lods,
                const cadr_view* view, cadr_draw_indexed_cmd* cmds, uint32_t* counts,
                uint32_t* marginal, float* world, float* world_sphere, int threads)
{
    if (L < 1 || L > 4 || check_offsets(n, S, off)) return -1;
    set_threads(threads);
    int rc = 0;
    /* Internal levels, top down: level 0's world is its local matrix. */
    float* prev = NULL;
    uint64_t prev_n = 0;
    for (uint32_t l = 0; l < num_levels && rc == 0; l++) {
        float* w = (float*)malloc(level_size[l] * 64 + 64);
        if (!w) {
            rc = -1;
            break;
        }
        if (l == 0)
            memcpy(w, level_local[0], level_size[0] * 64);
        else
            rc = oracle_propagate(prev, prev_n, level_local[l], level_parent[l], level_size[l], w,
                                  threads);
        free(prev);
        prev = w;
        prev_n = level_size[l];
    }
    float* wm = world ? world : (float*)malloc(n * 64 + 64);
    float* ws = world_sphere ? world_sphere : (float*)malloc(n * 16 + 16);
    if (!wm || !ws) rc = -1;
    if (rc == 0)
        rc = oracle_propagate(prev, prev_n, local, num_levels ? parent : NULL, n, wm, threads);
    if (rc == 0) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++)
            oracle_sphere_transform(wm + 16 * i, sphere + 4 * i, ws + 4 * i);
        rc = oracle_cull_spheres(n, ws, geometry, S, off, G, L, lods, view, cmds, counts, marginal,
                                 threads);
    }
    free(prev);
    if (!world) free(wm);
    if (!world_sphere) free(ws);
    return rc;
}

/* StateSet::prepareRecording counts each StateSet's drawables
 * (StateSet.cpp:180-195); recordToCommandBuffer then copies each list at
 * drawableCounter and advances it, StateSet by StateSet in depth-first
 * order (StateSet.cpp:198-268).  The lists are rebuilt here from the
 * (StateSet, list index) of every slot. */
int oracle_pack_state_sets(uint32_t S, const uint32_t* dfs_order, uint64_t n, const uint32_t* state_set_of_slot,
                           const uint32_t* list_index_of_slot, const cadr_drawable_gpu_data* pool,
                           cadr_drawable_gpu_data* packed, uint32_t* offsets)
{
    int rc = 0;
    uint64_t* count = (uint64_t*)calloc(S ? S : 1, sizeof(uint64_t));
    uint64_t* first = (uint64_t*)calloc(S ? S : 1, sizeof(uint64_t));
    uint8_t* seen_set = (uint8_t*)calloc(S ? S : 1, 1);
    uint64_t* list = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
    uint8_t* used = (uint8_t*)calloc(n ? n : 1, 1);
    if (!count || !first || !seen_set || !list || !used) {
        rc = -1;
        goto done;
    }
    for (uint32_t j = 0; j < S; j++) {
        if (dfs_order[j] >= S || seen_set[dfs_order[j]]) {
            rc = -1;
            goto done;
        }
        seen_set[dfs_order[j]] = 1;
    }
    for (uint64_t k = 0; k < n; k++) {
        if (state_set_of_slot[k] >= S) {
            rc = -1;
            goto done;
        }
        count[state_set_of_slot[k]]++;
    }
    /* the lists, StateSet after StateSet in id order */
    {
        uint64_t run = 0;
        for (uint32_t s = 0; s < S; s++) {
            first[s] = run;
            run += count[s];
        }
    }
    for (uint64_t k = 0; k < n; k++) {
        const uint32_t s = state_set_of_slot[k];
        const uint64_t li = list_index_of_slot[k];
        if (li >= count[s] || used[first[s] + li]) {
            rc = -1;
            goto done;
        }
        used[first[s] + li] = 1;
        list[first[s] + li] = k;
    }
    /* recordToCommandBuffer: drawableCounter over the depth-first order */
    {
        uint64_t drawable_counter = 0;
        for (uint32_t j = 0; j < S; j++) {
            const uint32_t s = dfs_order[j];
            offsets[j] = (uint32_t)drawable_counter;
            for (uint64_t li = 0; li < count[s]; li++) packed[drawable_counter + li] = pool[list[first[s] + li]];
            drawable_counter += count[s];
        }
        offsets[S] = (uint32_t)drawable_counter;
    }
done:
    free(count);
    free(first);
    free(seen_set);
    free(list);
    free(used);
    return rc;
}

/* ---- vertex-pulling consumer check (examples/RenderingPerformance/shader.vert:100-120) ---- */

static int region_find(const oracle_region* r, uint32_t nr, uint64_t addr, uint64_t bytes, uint64_t align,
                       const uint8_t** p)
{
    if (addr % align) return 0;
    for (uint32_t k = 0; k < nr; k++) {
        const uint64_t end = r[k].base + r[k].size;
        if (addr >= r[k].base && addr <= end && bytes <= end - addr) {
            *p = r[k].bytes + (addr - r[k].base);
            return 1;
        }
    }
    return 0;
}

static uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint32_t fbits32(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}

static uint64_t pair32(float lo, float hi) { return (uint64_t)fbits32(lo) | ((uint64_t)fbits32(hi) << 32); }

/* r = ((a0*b.x + a1*b.y) + a2*b.z) + a3*b.w, one rounding per operation */
static void col4(const float* a0, const float* a1, const float* a2, const float* a3, const float* b, float* r)
{
    for (int c = 0; c < 4; c++) {
        volatile float t0 = a0[c] * b[0], t1 = a1[c] * b[1], t2 = a2[c] * b[2], t3 = a3[c] * b[3];
        volatile float s0 = t0 + t1;
        volatile float s1 = s0 + t2;
        volatile float s2 = s1 + t3;
        r[c] = s2;
    }
}

static float mul(float a, float b)
{
    volatile float r = a * b;
    return r;
}
static float add(float a, float b)
{
    volatile float r = a + b;
    return r;
}
static float divf(float a, float b)
{
    volatile float r = a / b;
    return r;
}

int oracle_check_draws(const oracle_region* regions, uint32_t nr, const cadr_draw_indirect_cmd* indirect,
                       const cadr_drawable_pointers* pointers, uint64_t n, const cadr_consumer_view* v,
                       cadr_draw_check* out, int threads)
{
    const uint64_t K = 0x9E3779B97F4A7C15ull;
    const float* V = v->view;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int64_t d = 0; d < (int64_t)n; d++) {
        const cadr_draw_indirect_cmd cmd = indirect[d];
        const cadr_drawable_pointers dp = pointers[d];
        uint32_t flags = 0, pulled = 0;
        uint64_t sum = 0;
        const uint8_t* p;
        if (dp.drawable_data_ptr && !region_find(regions, nr, dp.drawable_data_ptr, 64, 64, &p))
            flags |= CADR_DRAW_BAD_DRAWABLE_DATA;
        const uint8_t* mlp;
        if (!region_find(regions, nr, dp.matrix_list_ptr, 64, 64, &mlp)) {
            flags |= CADR_DRAW_BAD_MATRIX_LIST;
        } else {
            uint32_t num_matrices;
            memcpy(&num_matrices, mlp, 4);
            for (uint64_t m = cmd.first_instance; m < (uint64_t)cmd.first_instance + cmd.instance_count; m++) {
                if (m >= num_matrices) {
                    flags |= CADR_DRAW_BAD_INSTANCE;
                    break;
                }
                const uint8_t* mp;
                if (!region_find(regions, nr, dp.matrix_list_ptr + 64 + 64 * m, 64, 16, &mp)) {
                    flags |= CADR_DRAW_BAD_MATRIX_LIST;
                    continue;
                }
                float M[16], W[16];
                memcpy(M, mp, 64);
                for (int c = 0; c < 4; c++) col4(V, V + 4, V + 8, V + 12, M + 4 * c, W + 4 * c);
                /* the GPU's lanes stop at their first bad index read; lane l
                 * reads k = l, l + 32, ... */
                for (uint32_t lane = 0; lane < 32; lane++) {
                    for (uint64_t k = lane; k < cmd.vertex_count; k += 32) {
                        const uint8_t* ip;
                        if (!region_find(regions, nr, dp.index_data_ptr + 4ull * ((uint64_t)cmd.first_vertex + k), 4, 4, &ip)) {
                            flags |= CADR_DRAW_BAD_INDEX_READ;
                            break;
                        }
                        uint32_t index;
                        memcpy(&index, ip, 4);
                        const uint8_t* vp;
                        if (!region_find(regions, nr, dp.vertex_data_ptr + 12ull * index, 12, 4, &vp)) {
                            flags |= CADR_DRAW_BAD_VERTEX_READ;
                            continue;
                        }
                        float pos[4];
                        memcpy(pos, vp, 12);
                        pos[3] = 1.0f;
                        float e[4];
                        col4(W, W + 4, W + 8, W + 12, pos, e);
                        const float gx = add(add(mul(v->p11, e[0]), mul(v->p31, e[2])), mul(v->p41, e[3]));
                        const float gy = add(add(mul(v->p22, e[1]), mul(v->p32, e[2])), mul(v->p42, e[3]));
                        const float gz = add(mul(v->p33, e[2]), mul(v->p43, e[3]));
                        const float gw = add(mul(v->p34, e[2]), mul(v->p44, e[3]));
                        const float ex = divf(e[0], e[3]), ey = divf(e[1], e[3]), ez = divf(e[2], e[3]);
                        sum += mix64(pair32(gx, gy)) ^ mix64(pair32(gz, gw) ^ K) ^ mix64(pair32(ex, ey) ^ (2 * K)) ^
                               mix64(((uint64_t)fbits32(ez) | ((uint64_t)index << 32)) ^ (3 * K));
                        pulled++;
                    }
                }
            }
        }
        out[d].checksum = sum;
        out[d].pulled = pulled;
        out[d].flags = flags;
    }
    return 0;
}
