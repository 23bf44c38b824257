// ref_host_shims.hpp — included by the translated host functions
// (oracle/_ref/ref_host.hpp) inside their namespace, after the translated
// structs.
//
// TEST INFRASTRUCTURE ONLY. SphSimulation3DGrid (src/simulation/
// sph_3d_grid.rs:33-101) owns wgpu pipelines and buffers; spawn_particles
// (:1534-1569) touches only the fields below, with the same names and types
// (its two wgpu buffers are host byte vectors here, see rs_runtime.hpp).
#pragma once

struct SphSimulation3DGrid {
  rs::Buffer particle_buffer;     // sph_3d_grid.rs:47
  rs::Buffer grid_params_buffer;  // :61
  GpuGridParams grid_params{};    // :98
  uint32_t num_particles{};       // :99
  uint32_t max_particles{};       // :100
};
