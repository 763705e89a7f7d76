// facade_glm_test.cpp - the facade's MatrixList and Geometry used as the
// reference's code uses them, with glm::mat4 (GLM on the include path):
// setMatrices() for one matrix and for a vector, editNewContent() filled in
// place, the Geometry getters and staging helpers.  Host-memory backend, no
// GPU.  Exits 0 on success.
#include <CadR/Geometry.h>
#include <CadR/MatrixList.h>
#include <CadR/Renderer.h>

#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include <glm/mat4x4.hpp>

using namespace CadR;

static int g_fail = 0;
#define EXPECT(c, msg)                                      \
    do {                                                    \
        if (!(c)) {                                         \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, msg); \
            g_fail = 1;                                     \
        }                                                   \
    } while (0)

// Host-memory backend: an allocation's device address is its host address.
static const uint8_t* at(uint64_t address) { return reinterpret_cast<const uint8_t*>(address); }

int main()
{
    static_assert(std::is_same<Mat4, glm::mat4>::value, "Mat4 is glm::mat4 with GLM on the include path");
    HostMemoryBackend be(16 << 20);
    Renderer r(be);
    r.beginFrame();

    glm::mat4 a(1.0f);
    a[3] = glm::vec4(1.f, 2.f, 3.f, 1.f);
    std::vector<glm::mat4> v(3, glm::mat4(2.0f));
    MatrixList m1(r), m2(r), m3(r);
    m1.setMatrices(a);
    m2.setMatrices(v);
    glm::mat4* e = m3.editNewContent(2);
    e[0] = glm::mat4(3.0f);
    e[1] = a;

    Geometry g(r);
    const float verts[9] = {0, 0, 0, 1, 0, 0, 0, 1, 0};
    const uint32_t idx[3] = {0, 1, 2};
    g.uploadVertexData(verts, sizeof(verts));
    StagingData sd = g.createIndexStagingData(sizeof(idx));
    std::memcpy(sd.data(), idx, sizeof(idx));
    PrimitiveSet ps{3, 0};
    g.uploadPrimitiveSetData(&ps, sizeof(ps));
    r.executeCopyOperations();

    uint32_t h[2];
    std::memcpy(h, at(m1.deviceAddress()), 8);
    EXPECT(h[0] == 1 && h[1] == 1 && std::memcmp(at(m1.deviceAddress()) + 64, &a, 64) == 0, "one matrix");
    std::memcpy(h, at(m2.deviceAddress()), 8);
    EXPECT(h[0] == 3 && std::memcmp(at(m2.deviceAddress()) + 64, v.data(), 3 * 64) == 0, "a vector of matrices");
    const glm::mat4 three(3.0f);
    std::memcpy(h, at(m3.deviceAddress()), 8);
    EXPECT(h[0] == 2 && std::memcmp(at(m3.deviceAddress()) + 64, &three, 64) == 0 &&
               std::memcmp(at(m3.deviceAddress()) + 128, &a, 64) == 0,
           "editNewContent");
    EXPECT(&g.renderer() == &r && &g.dataStorage() == &r.dataStorage(), "Geometry getters");
    EXPECT(g.vertexDataSize() == sizeof(verts) && g.indexDataSize() == sizeof(idx) &&
               g.primitiveSetDataSize() == sizeof(ps),
           "Geometry sizes");
    const Geometry& cg = g;
    EXPECT(std::memcmp(at(cg.indexDataAllocation().deviceAddress()), idx, sizeof(idx)) == 0,
           "index data staged and uploaded");
    // move assignment (DataAllocation.h:173, Geometry.h: operator=(Geometry&&))
    Geometry g2(r);
    const uint64_t vh = g.vertexDataAllocation().handle();
    g2 = std::move(g);
    EXPECT(g2.vertexDataSize() == sizeof(verts) && g2.vertexDataAllocation().handle() == vh &&
               g.vertexDataSize() == 0 && g.vertexDataAllocation().handle() == 0,
           "Geometry move assignment");
    DataAllocation d1(r.dataStorage()), d2(r.dataStorage());
    d2.upload(idx, sizeof(idx));
    const uint64_t h2 = d2.handle();
    d1 = std::move(d2);
    EXPECT(d1.handle() == h2 && d1.size() == sizeof(idx) && d2.handle() == 0 && d2.size() == 0,
           "DataAllocation move assignment");
    g2.freeData();
    EXPECT(g2.vertexDataSize() == 0 && g2.indexDataSize() == 0 && g2.primitiveSetDataSize() == 0, "freeData");
    if (!g_fail) std::printf("facade glm ok\n");
    return g_fail;
}
