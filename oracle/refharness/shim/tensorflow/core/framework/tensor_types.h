// Stand-in for the one TensorFlow type the reference's CUDA headers name:
// the launchers take an Eigen::GpuDevice, which the host harness never uses.
#pragma once
namespace Eigen { struct GpuDevice { void* stream() const { return nullptr; } }; }
