// tube-segmentation.hpp -- the library entry point of the Tube Segmentation
// Framework API (reference tube-segmentation.hpp:47).
//
//   TSFOutput *run(std::string filename, paramList &parameters, std::string kernel_dir);
//   TSFOutput *runSegmentation(...)   -- the same call under the name the
//                                        benchmark description uses
//
// run() reads an .mhd/.raw volume, crops it (`cropping lung|threshold`; the
// AAA-Vessels-CT preset's in-plane crop; else a shrink of every extent to a
// multiple of 4; getShiftVector() gives the box corner), converts it to [0,1]
// floats, and runs the
// GPU hot path of the `gpu` centerline method on the current CUDA device:
// Gaussian blur, the vector field, the small-radius TDF on the un-diffused
// field, GVF (Jacobi, or full multigrid with use-fmg-gvf), the large-radius
// TDF (circle fitting, or the spline TDF with use-spline-tdf) and the
// combination of both, then the candidate stage (threshold,
// compaction, cross-section filter, per-cube arg-max).  kernel_dir is
// accepted and ignored (the kernels are compiled into the library).
//
// Results: the TDF always; with `tdf-only` nothing else.  With
// `centerpoints-only` the centerline voxels are the filtered candidate mask,
// exactly the reference's output for that option.  Otherwise getCenterpoints()
// lists the centerpoint vertices, the vertices are linked into trees and the
// centerline voxels are the rasterised large trees (after loop removal with
// `loop-removal` or a `centerline-vtk-file`, which is also written).  Unless
// `no-segmentation` is set, the segmentation follows: inverse-gradient region
// growing from the centerlines, or spheres of the TDF radius with
// `sphere-segmentation`.
//
// Exceptions follow the reference: SIPL::IOException for a missing file,
// SIPL::SIPLException for a bad header, an unsupported type or option, or a
// candidate / vertex count outside the accepted range.
#ifndef TSF_TUBE_SEGMENTATION_HPP
#define TSF_TUBE_SEGMENTATION_HPP

#include <string>

#include "tsf/SIPL/Exceptions.hpp"
#include "tsf/SIPL/Types.hpp"
#include "tsf/inputOutput.hpp"
#include "tsf/parameters.hpp"

TSFOutput *run(std::string filename, paramList &parameters, std::string kernel_dir);
TSFOutput *runSegmentation(std::string filename, paramList &parameters, std::string kernel_dir);

#endif
