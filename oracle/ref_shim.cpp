// ref_shim.cpp - exposes the CADR reference's own sphere and matrix math
// (src/CadR/BoundingSphere.h:70-86 and GLM's mat4 operator*, as used by
// examples/gltfReader/main.cpp:1546) through a C interface, so the oracle's
// restatement can be checked against the reference code itself.
//
// TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` from the
// reference sources where they lie; the result goes to oracle/_ref/ and is
// used by the CPU tests and by tests/golden/make_golden.py.
#include <CadR/BoundingSphere.h>
#include <glm/mat4x4.hpp>
#include <cstring>

extern "C" {

__attribute__((visibility("default"))) void ref_mat4_mul(const float* a, const float* b,
                                                          float* out)
{
    glm::mat4 A, B;
    std::memcpy(&A, a, 64);
    std::memcpy(&B, b, 64);
    glm::mat4 R = A * B;
    std::memcpy(out, &R, 64);
}

__attribute__((visibility("default"))) void ref_sphere_transform(const float* m,
                                                                  const float* s, float* out)
{
    glm::mat4 M;
    std::memcpy(&M, m, 64);
    CadR::BoundingSphere bs{glm::vec3(s[0], s[1], s[2]), s[3]};
    CadR::BoundingSphere r = M * bs;
    out[0] = r.center.x;
    out[1] = r.center.y;
    out[2] = r.center.z;
    out[3] = r.radius;
}

__attribute__((visibility("default"))) int ref_glm_version() { return GLM_VERSION; }
}
