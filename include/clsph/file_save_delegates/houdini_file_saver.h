// Houdini frame writer of libclsph/file_save_delegates/houdini_file_saver.h:8-20:
// every call writes <prefix>frames/frameNNNNNNN.geo (7-digit counter starting
// at 1), the ASCII PGEOMETRY V5 format of
// libclsph/file_save_delegates/houdini_file_saver.cpp:28-74.
//
// The reference switches to a binary .bgeo frame through Partio when it is
// compiled with USE_PARTIO (houdini_file_saver.cpp:76-88 with the attributes of
// util/partio/PartioFunctions.h:5-65). Here the binary writer is part of the
// library (no Partio needed): code compiled with -DUSE_PARTIO gets savers that
// write <prefix>frames/frameNNNNNNN.bgeo, and any saver can be switched with
// the `binary_bgeo` member.
#ifndef _HOUDINI_FILE_SAVER_H_
#define _HOUDINI_FILE_SAVER_H_

#include <string>

#include "common/structures.h"

class houdini_file_saver {
 public:
  houdini_file_saver(std::string frames_folder_prefix)
      : frames_folder_prefix(frames_folder_prefix),
#ifdef USE_PARTIO
        binary_bgeo(true),
#else
        binary_bgeo(false),
#endif
        frame_count(0) {
  }

  int writeFrameToFile(particle* particles, const simulation_parameters& parameters);

  std::string frames_folder_prefix;
  // true: classic binary Houdini geometry (.bgeo) with Partio's attribute set;
  // false: the ASCII .geo file.
  bool binary_bgeo;

 private:
  int frame_count;
};

#endif
