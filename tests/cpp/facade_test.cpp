// facade_test.cpp - tests of the C++ facade (include/CadR).
//
//   facade_test cpu   host-memory backend, no GPU:
//     * the allocator placement checks of the reference's
//       tests/DataAllocationTest.cpp (first allocation at the block start,
//       zero size at address 0, spacing 16/32/48/64/128/(s+63)&~63, memory
//       empty after six free orders, wrap-around through block 2), over a
//       subset of its (size, count) ranges;
//     * HandleTable growth to 2 and 3 levels and table walks as the shader
//       does them;
//     * StateSet depth-first packing, swap-remove and draw calls, with the
//       oracle run over the host arena;
//     * the StateSet child and parent lists: both sides linked by one
//       append, unlinked by one remove, iteration both ways, destruction
//       detaching an object from its parents and children;
//     * Drawable create / move / getters and StateSet's drawable functions;
//     * FrameInfo's CPU timestamps;
//   facade_test gpu   the CUDA Renderer: processDrawables on the device,
//     compared word for word with the oracle over the downloaded blocks;
//     the device-resident path frame by frame against the copying path
//     (drawables and the StateSet tree changing between frames); FrameInfo's
//     GPU timestamps.
// Exits 0 on success, prints the first failure otherwise.
#include <CadR/Renderer.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../oracle/cadr_oracle.h"

using namespace CadR;

static int g_fail = 0;
#define EXPECT(c, ...)                                  \
    do {                                                \
        if (!(c)) {                                     \
            std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
            std::printf(__VA_ARGS__);                   \
            std::printf("\n");                          \
            g_fail = 1;                                 \
            return;                                     \
        }                                               \
    } while (0)

static bool storage_empty(const DataStorage& ds)
{
    for (const DataMemory* m : ds.dataMemoryList()) {
        if (m->usedBytes() != 0 || !m->empty()) return false;
        if (m->block1Start() != m->deviceAddress() || m->block1End() != m->deviceAddress()) return false;
        if (m->block2End() != m->deviceAddress()) return false;
    }
    return true;
}

static size_t spacing(size_t s)
{
    return (s == 0) ? 0 : (s <= 16) ? 16 : (s <= 32) ? 32 : (s <= 48) ? 48 : (s <= 64) ? 64 : (s <= 128) ? 128 : (s + 63) & ~size_t(63);
}

// tests/DataAllocationTest.cpp:55-326, the same sequence of checks.
static void test_allocation_placement()
{
    HostMemoryBackend be(64 << 20);
    Renderer r(be);
    DataStorage& ds = r.dataStorage();
    EXPECT(storage_empty(ds), "fresh storage not empty");
    HandlelessAllocation a(ds);
    a.alloc(10);
    DataMemory& m = *ds.dataMemoryList().front();
    const uint64_t first = a.deviceAddress();
    EXPECT(first == m.deviceAddress(), "first allocation not at the block start");
    EXPECT(m.size() == DataStorage::smallMemorySize, "first block is not 64 KiB");
    a.free();
    a.free();
    r.executeCopyOperations();
    EXPECT(storage_empty(ds), "not empty after free");
    a.alloc(10);
    EXPECT(a.deviceAddress() == m.deviceAddress(), "re-allocation not at the block start");
    r.executeCopyOperations();
    a.free();
    a.free();
    EXPECT(storage_empty(ds), "not empty after second free");
    a.alloc(0);
    EXPECT(a.deviceAddress() == 0, "zero-size allocation address is not 0");
    a.free();
    EXPECT(storage_empty(ds), "not empty after zero-size free");
    for (size_t s = 0; s < 260; s++) {
        a.alloc(s);
        EXPECT(a.deviceAddress() == first || (a.deviceAddress() == 0 && s == 0), "size %zu not at start", s);
        a.free();
        r.executeCopyOperations();
        EXPECT(storage_empty(ds), "size %zu: not empty", s);
    }
    for (int order = 0; order < 2; order++) {
        for (size_t s = 0; s < 260; s++) {
            HandlelessAllocation a1(ds), a2(ds);
            a1.alloc(s);
            a2.alloc(s);
            EXPECT(a1.deviceAddress() == first || (a1.deviceAddress() == 0 && s == 0), "a1 size %zu", s);
            EXPECT(a2.deviceAddress() == first + spacing(s) || (a2.deviceAddress() == 0 && s == 0),
                   "a2 size %zu at +%lld, want +%zu", s, (long long)(a2.deviceAddress() - first), spacing(s));
            if (order == 0) {
                a1.free();
                a2.free();
            } else {
                a2.free();
                a1.free();
            }
            r.executeCopyOperations();
            EXPECT(storage_empty(ds), "pair size %zu order %d: not empty", s, order);
        }
    }
    const size_t sizes[] = {0, 1, 10, 15, 16, 17, 31, 32, 33, 47, 48, 49, 63, 64, 65, 100, 127, 128, 129, 200, 259};
    const size_t counts[] = {0, 1, 2, 3, 5, 8, 31, 100, 255, 256, 395, 396, 511, 512, 1000, 1029};
    for (size_t s : sizes) {
        const size_t off = spacing(s);
        for (size_t n : counts) {
            if (off * n >= 65536) continue;
            std::vector<HandlelessAllocation> v;
            v.reserve(1030);
            auto fill = [&](size_t k) {
                for (size_t i = 0; i < k; i++) v.emplace_back(ds).alloc(s);
            };
            auto done = [&](const char* what) -> bool {
                v.clear();
                r.executeCopyOperations();
                if (!storage_empty(ds)) {
                    std::printf("FAIL: size %zu count %zu: not empty after %s\n", s, n, what);
                    g_fail = 1;
                    return false;
                }
                return true;
            };
            fill(n);
            for (size_t i = 0; i < n; i++)
                EXPECT(v[i].deviceAddress() == first + off * i || (v[i].deviceAddress() == 0 && s == 0),
                       "size %zu count %zu index %zu misplaced", s, n, i);
            for (size_t i = 0; i < n; i++) v[i].free();
            if (!done("in-order free")) return;
            fill(n);
            for (size_t i = n; i > 0;) v[--i].free();
            if (!done("reverse free")) return;
            fill(n);
            for (size_t i = 0; i < n; i += 2) v[i].free();
            for (size_t i = 1; i < n; i += 2) v[i].free();
            if (!done("even-then-odd free")) return;
            fill(n);
            for (size_t i = 1; i < n; i += 2) v[i].free();
            for (size_t i = 0; i < n; i += 2) v[i].free();
            if (!done("odd-then-even free")) return;
            fill(n);
            for (int64_t i = int64_t(n) - 2; i >= 0; i -= 2) v[i].free();
            for (int64_t i = int64_t(n) - 1; i >= 0; i -= 2) v[i].free();
            if (!done("reverse every-second free")) return;
            fill(n);
            for (int64_t i = int64_t(n) - 1; i >= 0; i -= 2) v[i].free();
            for (int64_t i = int64_t(n) - 2; i >= 0; i -= 2) v[i].free();
            if (!done("reverse every-second free (2)")) return;
            // Block 1 at the end of the buffer, later allocations wrap to block 2.
            for (int rev = 0; rev < 2; rev++) {
                HandlelessAllocation big(ds);
                big.alloc(65536 - s);
                if (n != 0) v.emplace_back(ds).alloc(s);
                big.free();
                for (size_t i = 1; i < n; i++) v.emplace_back(ds).alloc(s);
                if (!rev)
                    for (size_t i = 0; i < n; i++) v[i].free();
                else
                    for (size_t i = n; i > 0;) v[--i].free();
                if (!done("block-1 sequence")) return;
            }
        }
    }
}

// Walks the tables in host memory exactly as processDrawables.comp:77-89.
static uint64_t walk(unsigned level, uint64_t root, uint64_t h)
{
    auto rd = [](uint64_t a) { return *reinterpret_cast<const uint64_t*>(a); };
    if (level == 1) return rd(root + 8ull * uint32_t(h));
    if (level == 2) return rd(rd(root + 8ull * uint32_t(h >> 11)) + 8ull * (uint32_t(h) & 0x7ff));
    const uint64_t t2 = rd(root + 8ull * uint32_t(h >> 22));
    return rd(rd(t2 + 8ull * (uint32_t(h >> 11) & 0x7ff)) + 8ull * (uint32_t(h) & 0x7ff));
}

static void test_handle_table()
{
    HostMemoryBackend be(256 << 20);
    Renderer r(be);
    DataStorage& ds = r.dataStorage();
    EXPECT(ds.handleLevel() == 0 && ds.handleTableDeviceAddress() == 0, "empty table");
    uint64_t h = 0;
    auto grow = [&](uint64_t upto) {
        while (h < upto) {
            h = ds.createHandle();
            ds.setHandle(h, 0x100000ull + h * 16);
        }
    };
    grow(2047);
    EXPECT(ds.handleLevel() == 1, "level %u at 2047", ds.handleLevel());
    grow(2048);
    EXPECT(ds.handleLevel() == 2, "level %u at 2048", ds.handleLevel());
    grow(2048ull * 2048 - 1);
    EXPECT(ds.handleLevel() == 2, "level %u at 2048^2-1", ds.handleLevel());
    grow(2048ull * 2048 + 3000);
    EXPECT(ds.handleLevel() == 3, "level %u past 2048^2", ds.handleLevel());
    r.executeCopyOperations();
    const uint64_t root = ds.handleTableDeviceAddress();
    for (uint64_t k = 1; k <= h; k += (k < 5000 ? 1 : 977)) {
        const uint64_t got = walk(3, root, k);
        EXPECT(got == 0x100000ull + k * 16, "handle %llu resolves to %llx", (unsigned long long)k, (unsigned long long)got);
    }
    EXPECT(walk(3, root, 0) == 0, "handle 0 must resolve to 0");
}

struct SceneBuild {
    std::vector<std::unique_ptr<Geometry>> geometries;
    std::vector<std::unique_ptr<MatrixList>> lists;
    std::vector<std::unique_ptr<DataAllocation>> data;
    std::vector<Drawable> drawables;
    std::unique_ptr<StateSet> root, a, b, c, d;
};

// Root with children A, B (empty), C; C has child D.  Drawables spread over
// root, A, C, D; every 7th is removed again (swap-remove).
static void build_scene(Renderer& r, SceneBuild& S, int nGeom, int nDraw)
{
    S.root = std::make_unique<StateSet>(r);
    S.a = std::make_unique<StateSet>(r);
    S.b = std::make_unique<StateSet>(r);
    S.c = std::make_unique<StateSet>(r);
    S.d = std::make_unique<StateSet>(r);
    S.root->appendChild(*S.a);
    S.root->appendChild(*S.b);
    S.root->appendChild(*S.c);
    S.c->appendChild(*S.d);
    for (int g = 0; g < nGeom; g++) {
        auto geo = std::make_unique<Geometry>(r);
        std::vector<float> verts(12 + g % 5, 1.0f);
        std::vector<uint32_t> idx(36, uint32_t(g));
        PrimitiveSet ps[3] = {{uint32_t(36 + g), uint32_t(g * 3)}, {uint32_t(12 + g % 7), 5}, {uint32_t(3), uint32_t(g)}};
        geo->uploadVertexData(verts.data(), verts.size() * 4);
        geo->uploadIndexData(idx.data(), idx.size() * 4);
        geo->uploadPrimitiveSetData(ps, sizeof(ps));
        S.geometries.push_back(std::move(geo));
    }
    StateSet* sets[4] = {S.root.get(), S.a.get(), S.c.get(), S.d.get()};
    S.drawables.reserve(nDraw);
    for (int i = 0; i < nDraw; i++) {
        auto ml = std::make_unique<MatrixList>(r);
        std::vector<Mat4> m(1 + i % 3);
        for (auto& x : m) x.fill(float(i));
        ml->setMatrices(m);
        Geometry& g = *S.geometries[(i * 7) % nGeom];
        StateSet& ss = *sets[((uint32_t(i) * 2654435761u) >> 7) % 4];
        const uint32_t off = uint32_t(8 * (i % 3));
        if (i % 4 == 0) {
            auto dd = std::make_unique<DataAllocation>(r.dataStorage());
            uint32_t payload[4] = {uint32_t(i), 1, 2, 3};
            dd->upload(payload, sizeof(payload));
            S.drawables.emplace_back(g, off, *ml, *dd, ss);
            S.data.push_back(std::move(dd));
        } else {
            S.drawables.emplace_back(g, off, *ml, ss);
        }
        S.lists.push_back(std::move(ml));
    }
    for (int i = 0; i < nDraw; i += 7) S.drawables[i].destroy();
}

static void test_recording_and_oracle()
{
    HostMemoryBackend be(256 << 20);
    Renderer r(be);
    SceneBuild S;
    r.beginFrame();
    build_scene(r, S, 50, 3000);
    const size_t n = r.prepareSceneRendering(*S.root);
    size_t live = 0;
    for (auto& d : S.drawables) live += d.isValid();
    EXPECT(n == live, "prepareRecording counted %zu, %zu live", n, live);
    std::vector<DrawCall> calls;
    r.recordSceneRendering(*S.root, calls);
    r.executeCopyOperations();
    // DFS order root, A, (B skipped: empty), C, D; regions back to back.
    const StateSet* order[4] = {S.root.get(), S.a.get(), S.c.get(), S.d.get()};
    EXPECT(calls.size() == 4, "%zu draw calls", calls.size());
    uint64_t expect_first = 0;
    for (size_t k = 0; k < calls.size(); k++) {
        EXPECT(calls[k].stateSet == order[k], "draw call %zu is the wrong StateSet", k);
        EXPECT(calls[k].first == expect_first, "draw call %zu first %llu", k, (unsigned long long)calls[k].first);
        EXPECT(calls[k].count == order[k]->getNumDrawables(), "draw call %zu count", k);
        EXPECT(calls[k].indirectOffset == expect_first * 16, "indirect offset");
        EXPECT(calls[k].drawablePointers == r.drawablePointersBufferAddress() + expect_first * 32, "pointers address");
        EXPECT(std::memcmp(r.drawableStagingData() + expect_first, order[k]->drawableDataList().data(),
                           calls[k].count * sizeof(DrawableGpuData)) == 0, "packed records of call %zu", k);
        expect_first += calls[k].count;
    }
    // The oracle resolves the packed records through the tables in the arena.
    oracle_region reg{be.arena(), reinterpret_cast<uint64_t>(be.arena()), be.arenaBytes()};
    std::vector<cadr_draw_indirect_cmd> ind(n);
    std::vector<cadr_drawable_pointers> ptr(n);
    const int rc = oracle_process_drawables_regions(&reg, 1, r.dataStorage().handleLevel(), r.dataStorage().handleTableDeviceAddress(),
                                                    reinterpret_cast<const cadr_drawable_gpu_data*>(r.drawableStagingData()),
                                                    n, ind.data(), ptr.data(), 1);
    EXPECT(rc == 0, "oracle lookup left the arena");
    // Expected values from the objects themselves.
    size_t k = 0;
    for (const StateSet* ss : order) {
        for (const DrawableGpuData& g : ss->drawableDataList()) {
            const uint64_t ml = ptr[k].matrix_list_ptr;
            const uint32_t num = *reinterpret_cast<const uint32_t*>(ml);
            EXPECT(ind[k].instance_count == num && num >= 1 && num <= 3, "numMatrices %u", num);
            const uint64_t psAddr = 0;  // resolved below through the geometry that owns the handle
            (void)psAddr;
            bool found = false;
            for (auto& geo : S.geometries) {
                if (geo->primitiveSetDataAllocation().handle() != g.primitiveSetHandle) continue;
                const auto* ps = reinterpret_cast<const PrimitiveSet*>(geo->primitiveSetDataAllocation().deviceAddress() +
                                                                       g.primitiveSetOffset);
                EXPECT(ind[k].vertex_count == ps->indexCount && ind[k].first_vertex == ps->startIndex, "primitive set");
                EXPECT(ptr[k].vertex_data_ptr == geo->vertexDataAllocation().deviceAddress(), "vertex pointer");
                EXPECT(ptr[k].index_data_ptr == geo->indexDataAllocation().deviceAddress(), "index pointer");
                found = true;
            }
            EXPECT(found, "geometry of record %zu", k);
            EXPECT(ind[k].first_instance == 0, "baseInstance");
            if (g.drawableDataHandle == 0) EXPECT(ptr[k].drawable_data_ptr == 0, "drawable data of handle 0");
            k++;
        }
    }
}

static void test_gpu()
{
    Renderer r(0);
    SceneBuild S;
    r.beginFrame();
    build_scene(r, S, 300, 20000);
    std::vector<DrawCall> calls;
    r.processDrawables(*S.root, calls);
    cadr_context* ctx = r.context();
    check(cadr_context_synchronize(ctx), "sync");
    size_t n = 0;
    for (auto& c : calls) n += c.count;
    std::vector<cadr_draw_indirect_cmd> gi(n), oi(n);
    std::vector<cadr_drawable_pointers> gp(n), op(n);
    check(cadr_download(ctx, gi.data(), reinterpret_cast<void*>(r.drawIndirectBufferAddress()), n * 16, nullptr), "dl");
    check(cadr_download(ctx, gp.data(), reinterpret_cast<void*>(r.drawablePointersBufferAddress()), n * 32, nullptr), "dl");
    // Download every DataMemory block and let the oracle walk them.
    std::vector<std::vector<uint8_t>> blocks;
    std::vector<oracle_region> regs;
    for (const DataMemory* m : r.dataStorage().dataMemoryList()) {
        blocks.emplace_back(m->size());
        check(cadr_download(ctx, blocks.back().data(), reinterpret_cast<void*>(m->deviceAddress()), m->size(), nullptr), "dl");
    }
    check(cadr_stream_synchronize(cadr_context_stream(ctx)), "sync");
    size_t bi = 0;
    for (const DataMemory* m : r.dataStorage().dataMemoryList())
        regs.push_back(oracle_region{blocks[bi++].data(), m->deviceAddress(), m->size()});
    const int rc = oracle_process_drawables_regions(regs.data(), uint32_t(regs.size()), r.dataStorage().handleLevel(),
                                                    r.dataStorage().handleTableDeviceAddress(),
                                                    reinterpret_cast<const cadr_drawable_gpu_data*>(r.drawableStagingData()),
                                                    n, oi.data(), op.data(), 4);
    EXPECT(rc == 0, "oracle lookup left the device blocks");
    EXPECT(std::memcmp(gi.data(), oi.data(), n * 16) == 0, "indirect commands differ from the oracle");
    EXPECT(std::memcmp(gp.data(), op.data(), n * 32) == 0, "drawable pointers differ from the oracle");
    EXPECT(r.dataStorage().handleLevel() == 2, "expected a two-level table, got %u", r.dataStorage().handleLevel());
    std::printf("gpu: %zu drawables in %zu draw calls, handle level %u, %zu device blocks\n", n, calls.size(),
                r.dataStorage().handleLevel(), regs.size());
}

// Indirect commands and DrawablePointers of the last processed frame.
static void download_frame(Renderer& r, size_t n, std::vector<cadr_draw_indirect_cmd>& ind,
                           std::vector<cadr_drawable_pointers>& ptr)
{
    cadr_context* ctx = r.context();
    check(cadr_context_synchronize(ctx), "sync");
    ind.assign(n, cadr_draw_indirect_cmd{});
    ptr.assign(n, cadr_drawable_pointers{});
    check(cadr_download(ctx, ind.data(), reinterpret_cast<void*>(r.drawIndirectBufferAddress()), n * 16, nullptr), "dl");
    check(cadr_download(ctx, ptr.data(), reinterpret_cast<void*>(r.drawablePointersBufferAddress()), n * 32, nullptr), "dl");
    check(cadr_stream_synchronize(cadr_context_stream(ctx)), "sync");
}

static bool same_calls(const std::vector<DrawCall>& a, const std::vector<DrawCall>& b)
{
    if (a.size() != b.size()) return false;
    for (size_t k = 0; k < a.size(); k++)
        if (a[k].stateSet != b[k].stateSet || a[k].first != b[k].first || a[k].count != b[k].count ||
            a[k].drawablePointers != b[k].drawablePointers || a[k].indirectOffset != b[k].indirectOffset)
            return false;
    return true;
}

// Device-resident recording against the copying path, frame by frame:
// same draw calls, same buffers; new drawables and removals between frames;
// a frame without changes launches nothing but processDrawables.
// The child and parent lists (CadR/ParentChildList.h) over StateSets of a
// renderer that never touches the device.
static void test_parent_child_lists()
{
    Renderer r(0);
    StateSet a(r), b(r), c(r);
    EXPECT(a.childList.empty() && a.childList.size() == 0, "fresh child list not empty");
    auto ab = a.childList.append(b);
    a.childList.append(c);
    EXPECT(a.childList.size() == 2 && &a.childList.front() == &b && &a.childList.back() == &c, "children of a");
    EXPECT(b.parentList.size() == 1 && &b.parentList.front() == &a, "parent of b");
    EXPECT(&*ab == &b && &ab->renderer() == &r, "iterator of the appended child");
    std::vector<StateSet*> fwd, rev;
    for (StateSet& x : a.childList) fwd.push_back(&x);
    for (auto it = a.childList.rbegin(); it != a.childList.rend(); ++it) rev.push_back(&*it);
    EXPECT(fwd == std::vector<StateSet*>({&b, &c}) && rev == std::vector<StateSet*>({&c, &b}), "iteration order");
    // a parent appended from the child's side shows in the parent's children
    c.parentList.append(b);
    EXPECT(b.childList.size() == 1 && &b.childList.front() == &c && c.parentList.size() == 2 &&
               &c.parentList.back() == &b, "append from the child's side");
    a.childList.remove(ab);
    EXPECT(a.childList.size() == 1 && b.parentList.empty(), "remove unlinks both sides");
    {
        StateSet d(r);
        c.childList.append(d);
        d.childList.append(a);
        EXPECT(c.childList.size() == 1 && a.parentList.size() == 1, "links to d");
    }
    EXPECT(c.childList.empty() && a.parentList.empty(), "destroying d detaches it from its parent and child");
    b.childList.clear();
    EXPECT(b.childList.empty() && c.parentList.size() == 1 && &c.parentList.front() == &a, "clear");
    const StateSet& ca = a;
    size_t k = 0;
    for (auto it = ca.childList.cbegin(); it != ca.childList.cend(); ++it) k++;
    EXPECT(k == 1, "const iteration");
    std::printf("parent/child lists ok\n");
}

// Drawable and StateSet drawable functions: create / move / getters,
// appendDrawable moving a drawable between StateSets, removeDrawable,
// removeAllDrawables, prepareCallList.
static void test_drawable_api()
{
    HostMemoryBackend be(16 << 20);
    Renderer r(be);
    Geometry g(r);
    MatrixList ml(r);
    ml.setMatrices(Mat4{});
    DataAllocation dd(r.dataStorage());
    dd.alloc(64);
    StateSet s1(r), s2(r);
    Drawable d1(g, 0, ml, s1), d2(g, 8, ml, dd, s1);
    EXPECT(s1.getNumDrawables() == 2 && &s1.getDrawable(0) == &d1 && &s1.getDrawable(1) == &d2, "two drawables in s1");
    EXPECT(&d2.matrixList() == &ml && d2.drawableData() == &dd && d1.drawableData() == nullptr && &d1.renderer() == &r,
           "getters");
    EXPECT(s1.drawableDataList()[1].drawableDataHandle == dd.handle() && s1.drawableDataList()[1].primitiveSetOffset == 8,
           "record of d2");
    s2.appendDrawable(d1, s1.drawableDataList()[0]);
    EXPECT(s1.getNumDrawables() == 1 && &s1.getDrawable(0) == &d2 && s2.getNumDrawables() == 1 && &d1.stateSet() == &s2,
           "appendDrawable moves d1 to s2");
    Drawable d3;
    d3 = std::move(d2);
    EXPECT(!d2.isValid() && d3.isValid() && &s1.getDrawable(0) == &d3 && d3.drawableData() == &dd, "move assignment");
    StateSet::removeDrawable(d3);
    EXPECT(!d3.isValid() && s1.getNumDrawables() == 0 && &d3.stateSet() == &s1, "removeDrawable");
    d3.create(g, 16, ml, s2);
    EXPECT(s2.getNumDrawables() == 2 && s2.drawableDataList()[1].primitiveSetOffset == 16, "create");
    s2.removeAllDrawables();
    EXPECT(!d1.isValid() && !d3.isValid() && s2.getNumDrawables() == 0, "removeAllDrawables");
    StateSet root(r), child(r);
    root.appendChild(child);
    int calls = 0;
    child.prepareCallList.push_back([&calls](StateSet& s) {
        calls++;
        s.requestRecording();
    });
    EXPECT(root.prepareRecording() == 0 && calls == 1, "prepareCallList");
    EXPECT(&Renderer::get() == &r, "the last renderer made default");
    {
        Renderer other(be, false);
        EXPECT(&Renderer::get() == &r, "makeDefault false leaves the default");
        Renderer::set(other);
        EXPECT(&Renderer::get() == &other, "Renderer::set");
    }
    Renderer::set(r);
    std::printf("drawable api ok\n");
}

// FrameInfo with the reference's fields: CPU timestamps in order on any
// backend; on the GPU the four GPU timestamps of a frame with drawable
// processing, in order, with a positive processing time.
static void check_cpu_times(const FrameInfo& f, const char* where)
{
    EXPECT(f.cpuBeginFrame <= f.cpuPrepareRecordingBegin && f.cpuPrepareRecordingBegin <= f.cpuPrepareRecordingEnd &&
               f.cpuPrepareRecordingEnd <= f.cpuRecordStateSetsBegin &&
               f.cpuRecordStateSetsBegin <= f.cpuRecordStateSetsEnd && f.cpuRecordStateSetsEnd <= f.cpuEndFrame &&
               f.gpuBeginFrame == f.cpuBeginFrame,
           "%s: CPU timestamps out of order", where);
}

// Renderer::finalize / leakResources / standardBufferAlignment
// (Renderer.cpp:89-94, 316-387; Renderer.h:228-229).
static void test_finalize()
{
    HostMemoryBackend be(256 << 20);
    Renderer r(be);
    SceneBuild S;
    r.beginFrame();
    build_scene(r, S, 20, 500);
    r.prepareSceneRendering(*S.root);
    std::vector<DrawCall> calls;
    r.recordSceneRendering(*S.root, calls);
    const size_t uploaded = r.executeCopyOperations();
    r.beginFrame();  // the previous frame's uploads become the staging hint (Renderer.cpp:394-397)
    EXPECT(uploaded > 0 && r.dataStorage().stagingDataSizeHint() == uploaded, "staging size hint %zu of %zu",
           r.dataStorage().stagingDataSizeHint(), uploaded);
    r.beginFrame();
    EXPECT(r.dataStorage().stagingDataSizeHint() == 0, "no uploads in the frame before");
    EXPECT(r.dataStorage().renderer() == &r, "DataStorage::renderer()");
    const size_t used = be.usedBlocks();
    EXPECT(r.drawableBufferAddress() && r.drawIndirectBufferAddress() && r.drawablePointersBufferAddress(),
           "drawable buffers allocated");
    r.finalize();
    EXPECT(be.usedBlocks() == used - 3, "finalize freed %zu of the 3 drawable buffers", used - be.usedBlocks());
    EXPECT(!r.drawableBufferAddress() && !r.drawIndirectBufferAddress() && !r.drawablePointersBufferAddress() &&
               r.drawableBufferSize() == 0,
           "buffers forgotten after finalize");
    r.finalize();  // idempotent
    EXPECT(be.usedBlocks() == used - 3, "a second finalize freed nothing more");
    EXPECT(r.standardBufferAlignment() == 256 && r.alignStandardBuffer(0) == 0 && r.alignStandardBuffer(1) == 256 &&
               r.alignStandardBuffer(256) == 256 && r.alignStandardBuffer(257) == 512,
           "standard buffer alignment");
    {
        // leakResources: the buffers stay allocated, the renderer forgets them
        HostMemoryBackend be2(64 << 20);
        Renderer r2(be2, false);
        SceneBuild S2;
        r2.beginFrame();
        build_scene(r2, S2, 5, 50);
        r2.prepareSceneRendering(*S2.root);
        std::vector<DrawCall> calls2;
        r2.recordSceneRendering(*S2.root, calls2);
        EXPECT(r2.drawableBufferAddress() != 0, "drawable buffers allocated");
        const size_t used2 = be2.usedBlocks();
        r2.leakResources();
        EXPECT(!r2.drawableBufferAddress() && be2.usedBlocks() == used2, "leakResources frees nothing");
    }
    if (!g_fail) std::printf("finalize ok\n");
}

// DataAllocation's construction forms, staging and handle functions
// (DataAllocation.h:54-96, 150-212; DataAllocation.cpp:18-51).
static void test_data_allocation_api()
{
    HostMemoryBackend be(16 << 20);
    Renderer r(be, false);
    DataStorage& ds = r.dataStorage();
    r.beginFrame();
    DataAllocation a = nullptr;  // implicit, as in CadR
    EXPECT(a.handle() == 0 && a.size() == 0, "an allocation of no storage");
    a.init(ds);
    EXPECT(a.handle() == 0 && &a.dataStorage() == &ds, "init binds the storage, no handle");
    struct Rec {
        uint32_t x, y;
    };
    a.setData(Rec{7, 9});
    Rec& e = a.editNewContent<Rec>();  // the same frame and size: the same staging
    e.y = 11;
    const uint64_t h = a.createHandle(ds);
    EXPECT(h != 0 && a.createHandle(ds) == h, "createHandle makes one handle");
    DataAllocation b(r, DataAllocation::noHandle);
    uint32_t* words = b.editNewContent<uint32_t>(4);
    for (uint32_t k = 0; k < 4; k++) words[k] = 100 + k;
    DataAllocation c(r);
    EXPECT(b.handle() == 0 && c.handle() != 0 && c.handle() != h, "handles");
    r.executeCopyOperations();
    const Rec* dev = reinterpret_cast<const Rec*>(a.deviceAddress());
    EXPECT(dev->x == 7 && dev->y == 11, "setData then editNewContent: %u %u", dev->x, dev->y);
    EXPECT(ds.handleLevel() == 1 &&
               reinterpret_cast<const uint64_t*>(ds.handleTableDeviceAddress())[h] == a.deviceAddress(),
           "the handle made after the data resolves to it");
    EXPECT(a.offset() == a.deviceAddress() - a.dataMemory().deviceAddress() && a.offset() < a.dataMemory().size(),
           "offset inside its DataMemory");
    EXPECT(&a.renderer() == &r, "renderer()");
    r.beginFrame();
    StagingData sd = b.alloc();  // a new frame: new content of the current size
    EXPECT(sd.size() == 16, "alloc() keeps the size");
    std::memset(sd.data(), 0xab, 16);
    EXPECT(sd.wasReallocated() && sd.sizeInBytes() == 16, "a new frame's content is new memory");
    StagingData again = b.createStagingData();
    EXPECT(again.data() == sd.data() && !again.wasReallocated(), "the frame's staging is reused");
    StagingData none;
    (void)none;
    r.executeCopyOperations();
    const uint8_t* bytes = reinterpret_cast<const uint8_t*>(b.deviceAddress());
    EXPECT(bytes[0] == 0xab && bytes[15] == 0xab, "alloc() content uploaded");
    a.destroyHandle();
    EXPECT(a.handle() == 0, "destroyHandle");
    // HandlelessAllocation: the same forms without a handle
    HandlelessAllocation u(nullptr), v(r);
    u.init(ds);
    u.setData(Rec{1, 2});
    v = std::move(u);
    EXPECT(v.size() == sizeof(Rec) && u.size() == 0 && &v.renderer() == &r, "handleless move assignment");
    r.executeCopyOperations();
    EXPECT(reinterpret_cast<const Rec*>(v.deviceAddress())->y == 2 && v.offset() < v.dataMemory().size(),
           "handleless content and offset");
    if (!g_fail) std::printf("data allocation api ok\n");
}

static void test_frame_info_host()
{
    HostMemoryBackend be(64 << 20);
    Renderer r(be);
    SceneBuild S;
    r.setCollectFrameInfo(true);
    r.beginFrame();
    build_scene(r, S, 8, 100);
    std::vector<DrawCall> calls;
    r.prepareSceneRendering(*S.root);
    r.recordSceneRendering(*S.root, calls);
    r.endFrame();
    const FrameInfo& f = r.getFrameInfo();
    EXPECT(f.frameNumber == ~size_t(0), "a frame without GPU timestamps reported as valid");
    check_cpu_times(f, "host frame");
    EXPECT(r.cpuTimestampPeriod() == 1e-9 && r.gpuTimestampPeriod() == 1e-9f, "timestamp periods");
    std::printf("frame info host ok\n");
}

static void test_gpu_frame_info()
{
    Renderer r(0);
    SceneBuild S;
    r.beginFrame();
    build_scene(r, S, 64, 20000);
    r.endFrame();
    r.setCollectFrameInfo(true);
    for (int k = 0; k < 3 && !g_fail; k++) {
        std::vector<DrawCall> calls;
        const size_t fn = r.beginFrame();
        if (k == 2)
            r.processDrawablesResident(*S.root, calls);
        else
            r.processDrawables(*S.root, calls);
        r.endFrame();
        const FrameInfo& f = r.getFrameInfo();
        EXPECT(f.frameNumber == fn, "frame %d: frameNumber %zu, expected %zu", k, f.frameNumber, fn);
        check_cpu_times(f, "gpu frame");
        EXPECT(f.gpuBeginExecution <= f.gpuAfterTransfersAndBeforeDrawableProcessing &&
                   f.gpuAfterTransfersAndBeforeDrawableProcessing < f.gpuAfterDrawableProcessingAndBeforeRendering &&
                   f.gpuAfterDrawableProcessingAndBeforeRendering <= f.gpuEndExecution,
               "frame %d: GPU timestamps out of order", k);
        const double ms = double(f.gpuAfterDrawableProcessingAndBeforeRendering -
                                 f.gpuAfterTransfersAndBeforeDrawableProcessing) * r.gpuTimestampPeriod() * 1e3;
        EXPECT(ms > 0.0 && ms < 100.0, "frame %d: drawable processing %.4f ms", k, ms);
    }
    r.setCollectFrameInfo(false);
    std::vector<DrawCall> calls;
    r.beginFrame();
    r.processDrawables(*S.root, calls);
    r.endFrame();
    EXPECT(r.getFrameInfo().frameNumber == ~size_t(0), "a frame without collection reported GPU timestamps");
    std::printf("gpu frame info ok\n");
}

static void test_gpu_resident()
{
    Renderer r(0);
    SceneBuild S;
    r.beginFrame();
    build_scene(r, S, 120, 12000);
    cadr_context* ctx = r.context();
    for (int frame = 0; frame < 5 && !g_fail; frame++) {
        if (frame == 1) {
            // Removals (swap-removes reorder the lists) and new drawables.
            for (size_t i = 3; i < S.drawables.size(); i += 11) S.drawables[i].destroy();
            StateSet* sets[3] = {S.a.get(), S.b.get(), S.d.get()};
            S.drawables.reserve(S.drawables.size() + 500);
            for (int i = 0; i < 500; i++) {
                auto ml = std::make_unique<MatrixList>(r);
                ml->setMatrices(std::vector<Mat4>(1 + i % 2));
                S.drawables.emplace_back(*S.geometries[i % S.geometries.size()], uint32_t(8 * (i % 3)), *ml, *sets[i % 3]);
                S.lists.push_back(std::move(ml));
            }
        }
        if (frame == 3) {
            // The tree alone changes: D moves from C to A.
            S.c->removeChild(*S.d);
            S.a->childList.append(*S.d);
        }
        std::vector<DrawCall> host, res;
        r.beginFrame();
        r.processDrawables(*S.root, host);
        size_t n = 0;
        for (auto& c : host) n += c.count;
        std::vector<cadr_draw_indirect_cmd> hi, ri;
        std::vector<cadr_drawable_pointers> hp, rp;
        download_frame(r, n, hi, hp);
        const uint64_t l0 = cadr_context_launch_count(ctx);
        r.processDrawablesResident(*S.root, res);
        const uint64_t launches = cadr_context_launch_count(ctx) - l0;
        download_frame(r, n, ri, rp);
        EXPECT(same_calls(host, res), "frame %d: draw calls differ", frame);
        EXPECT(std::memcmp(hi.data(), ri.data(), n * 16) == 0, "frame %d: indirect commands differ", frame);
        EXPECT(std::memcmp(hp.data(), rp.data(), n * 32) == 0, "frame %d: drawable pointers differ", frame);
        if (frame == 2 || frame == 4)
            EXPECT(launches == 1, "an unchanged frame launched %llu kernels", (unsigned long long)launches);
        if (frame == 3) EXPECT(launches > 1, "a tree change did not lay the pack out again");
        check(cadr_context_check_device_error(ctx, nullptr), "device error");
    }
    std::printf("gpu resident: 5 frames equal to the copying path\n");
}

int main(int argc, char** argv)
{
    const std::string mode = argc > 1 ? argv[1] : "cpu";
    try {
        if (mode == "cpu") {
            test_allocation_placement();
            if (!g_fail) test_handle_table();
            if (!g_fail) test_recording_and_oracle();
            if (!g_fail) test_parent_child_lists();
            if (!g_fail) test_drawable_api();
            if (!g_fail) test_frame_info_host();
            if (!g_fail) test_finalize();
            if (!g_fail) test_data_allocation_api();
        } else {
            test_gpu();
            if (!g_fail) test_gpu_resident();
            if (!g_fail) test_gpu_frame_info();
        }
    } catch (const std::exception& e) {
        std::printf("FAIL: exception %s\n", e.what());
        return 2;
    }
    if (!g_fail) std::printf("facade %s ok\n", mode.c_str());
    return g_fail;
}
