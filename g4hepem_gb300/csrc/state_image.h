// state_image.h -- host-side image of the device table arena.
#pragma once

#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include "tables.h"

namespace hepem {

struct StateImage {
  std::vector<uint8_t> bytes;                    // arena contents (256-byte aligned arrays)
  DevTables host;                                // pointer fields hold nothing useful yet
  std::vector<std::pair<size_t, size_t>> relocs; // (offset of pointer field in DevTables, arena offset)
};

// Parse + validate a G4HepEmState JSON document; throws std::runtime_error.
StateImage build_state_image(const char* text, size_t len);
StateImage build_state_image_file(const char* path);
// Binary image of a StateImage (serialize) and back (deserialize; throws
// std::runtime_error on a damaged or foreign image).
std::vector<uint8_t> serialize_image(const StateImage& img);
StateImage deserialize_image(const void* data, size_t size);
// Resolve the pointer fields against the arena base address `base`.
void relocate(StateImage& img, DevTables& out, const void* base);
// 64-bit FNV-1a hash (the checksum of the table image and of server snapshots).
uint64_t fnv1a(const uint8_t* p, size_t n);

}  // namespace hepem
