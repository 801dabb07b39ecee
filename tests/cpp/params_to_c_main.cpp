// Test driver for fluid_gb300::Params::to_c (host only, no device needed):
// the per-plane friction extension. Exit status 0 on success, else the
// number of the failed check.
#include "fluid_gb300.hpp"

int main() {
  fluid_gb300::Params p;
  p.planes.add(0.0f, 1.0f, 0.0f, 0.0f);
  p.planes.add(1.0f, 0.0f, 0.0f, 0.0f);
  fluid_params c = p.to_c();
  if (c.plane_count != 2 || c.plane_friction_per_plane != 0) return 1;
  p.plane_friction_each = {0.5f, 0.25f};
  c = p.to_c();
  if (c.plane_friction_per_plane != 1 || c.plane_friction_each[0] != 0.5f || c.plane_friction_each[1] != 0.25f)
    return 2;
  p.plane_friction_each = {0.5f};  // one value for two planes
  try {
    p.to_c();
    return 3;
  } catch (const fluid_gb300::Error& e) {
    if (e.status() != FLUID_ERR_INVALID_ARGUMENT) return 4;
  }
  return 0;
}
