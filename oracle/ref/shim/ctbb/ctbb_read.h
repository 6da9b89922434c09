/*
 * ctbb/ctbb_read.h (shim) -- declarations of the external libctbb_read readers
 * that the reference's src/setup.cu:31,418-475,693-752 calls.  The library is
 * absent and unpinned.  Only FileType 0 (float32 binary frames) is implemented
 * (ReadBinaryFrame, with frames past the end of the file read as zeros); the
 * vendor-format readers print an error and return zeros.
 *
 * TEST INFRASTRUCTURE: only used to build the reference CPU path in oracle/_ref.
 */
#ifndef CTBB_SHIM_CTBB_READ_H
#define CTBB_SHIM_CTBB_READ_H

#include <stdio.h>

void ReadBinaryFrame(FILE *fp, int frame_idx, int n_channels, int n_rows, float *frame,
                     int offset);

float ReadPTRTubeAngle(FILE *fp, int i, int n_channels, int n_rows);
float ReadPTRTablePosition(FILE *fp, int i, int n_channels, int n_rows);
void ReadPTRFrame(FILE *fp, int i, int n_channels, int n_rows, float *frame);

float ReadCTDv1794TubeAngle(FILE *fp, int i, int n_channels, int n_rows);
float ReadCTDv1794TablePosition(FILE *fp, int i, int n_channels, int n_rows);
void ReadCTDv1794Frame(FILE *fp, int i, int n_channels, int n_rows, float *frame);

float ReadCTDv2007TubeAngle(FILE *fp, int i, int n_channels, int n_rows);
float ReadCTDv2007TablePosition(FILE *fp, int i, int n_channels, int n_rows);
void ReadCTDv2007Frame(FILE *fp, int i, int n_channels, int n_rows, float *frame);

float ReadIMATubeAngle(FILE *fp, int i, int n_channels, int n_rows, int subtype, int offset);
float ReadIMATablePosition(FILE *fp, int i, int n_channels, int n_rows, int subtype, int offset);
void ReadIMAFrame(FILE *fp, int i, int n_channels, int n_rows, float *frame, int subtype,
                  int offset);

float ReadForceTubeAngle(FILE *fp, int i, int n_channels, int n_rows);
float ReadForceTablePosition(FILE *fp, int i, int n_channels, int n_rows);
void ReadForceFrame(FILE *fp, int i, int n_channels, int n_rows, float *frame);

float ReadDICOMTubeAngle(FILE *fp, int i, int n_channels, int n_rows);
float ReadDICOMTablePosition(FILE *fp, int i, int n_channels, int n_rows);
void ReadDICOMFrame(FILE *fp, int i, int n_channels, int n_rows, float *frame);

#endif
