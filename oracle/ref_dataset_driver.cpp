// Test driver (oracle side): runs the reference's own include/tsdfmc/dataset_io.h functions that work off
// Windows, printing floats as IEEE-754 hex words for bit comparison with the product's loader.
//   ref_dataset_driver pose <file>        -> R[9] t[3]
//   ref_dataset_driver intrinsics <file>  -> width height fx fy cx cy depth_scale (6 or 7 values only)
//   ref_dataset_driver frames <root>      -> frame ids
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "tsdfmc/dataset_io.h"

static unsigned hexf(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  const std::string cmd = argv[1];
  if (cmd == "pose") {
    const tsdfmc::Pose P = tsdfmc::loadPoseFromFile(argv[2]);
    for (int i = 0; i < 9; ++i) std::printf("%08x ", hexf(P.R.data[i]));
    std::printf("%08x %08x %08x\n", hexf(P.t.x), hexf(P.t.y), hexf(P.t.z));
  } else if (cmd == "intrinsics") {
    float scale = 0.0f;
    const tsdfmc::Intrinsics K = tsdfmc::loadDatasetIntrinsics(argv[2], scale);
    std::printf("%d %d %08x %08x %08x %08x %08x\n", K.width, K.height, hexf(K.fx), hexf(K.fy), hexf(K.cx), hexf(K.cy),
                hexf(scale));
  } else if (cmd == "frames") {
    for (int id : tsdfmc::listDatasetFrameIds(argv[2])) std::printf("%d\n", id);
  } else {
    return 2;
  }
  return 0;
}
