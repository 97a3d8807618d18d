// White-box check of fgb_sim_new's device rule: a simulation whose meshes
// belong to different CUDA devices is refused with FGB_EINVAL before any
// device work.  The test marks the second mesh as created on another device
// through the library's internal handle layout (handles.h), so it needs no
// GPU and launches nothing.
#include <cstdio>
#include <cstring>
#include <math.h>

#include "feriphys_gb300.h"
#include "handles.h"

static int fails = 0;
#define EXPECT(cond)                                           \
  do {                                                         \
    if (!(cond)) {                                             \
      std::printf("FAILED %s (line %d)\n", #cond, __LINE__); \
      ++fails;                                                 \
    }                                                          \
  } while (0)

int main() {
  const float pos[3] = {0, 0, 0};
  fgb_mesh* a = nullptr;
  fgb_mesh* b = nullptr;
  EXPECT(fgb_cloth_new(4, 4, 0.1f, pos, 0.01f, 1, 1, 1, 1, 1, 1, nullptr, 0, &a) == FGB_OK);
  EXPECT(fgb_cloth_new(4, 4, 0.1f, pos, 0.01f, 1, 1, 1, 1, 1, 1, nullptr, 0, &b) == FGB_OK);
  fgb_mesh* both[2] = {a, b};
  fgb_sim* s = nullptr;
  EXPECT(fgb_sim_new(both, 2, nullptr, 0, &s) == FGB_OK);  // same device: accepted
  fgb_sim_destroy(s);
  s = nullptr;
  b->device = a->device + 1;  // as if b had been created with another device current
  EXPECT(fgb_sim_new(both, 2, nullptr, 0, &s) == FGB_EINVAL);
  EXPECT(s == nullptr);
  EXPECT(std::strstr(fgb_last_error(), "one device") != nullptr);
  b->device = a->device;
  fgb_mesh_destroy(a);
  fgb_mesh_destroy(b);
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
