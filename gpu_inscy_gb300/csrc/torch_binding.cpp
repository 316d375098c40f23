// Python binding of the engine as a PyTorch C++ extension (module
// inscy_gb300_ext), with the entry points of the reference's own extension:
//
//   run_gpu_5(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells,
//             rectangular, entropy_order) -> [subspaces, clusterings]
//                                                      inscy_map.cpp:1070-1158
//   run_gpu_4(...same...)                              inscy_map.cpp:979-1067
//
// X is a float32 [n, d] tensor on the CPU or on a CUDA device; the result is
// the reference's pair of lists: one ascending dim list per clustered
// subspace and one label list (n ints) per subspace, in the reference's
// result-map order.  A CUDA tensor is read in place, with the work queued on
// the current CUDA stream of its device.  The extension only binds: every
// computation is the C ABI of libinscy_gb300.so (include/inscy_gb300.h).
// Failures raise RuntimeError with the engine's message, where the
// reference exits the process.
#include <torch/extension.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/inscy_gb300.h"

namespace {

std::vector<std::vector<std::vector<int>>> run(at::Tensor X, double neighborhood_size, double F, int64_t num_obj,
                                               int64_t min_size, double r, int64_t number_of_cells, bool rectangular,
                                               int64_t entropy_order, int mode) {
  TORCH_CHECK(X.dim() == 2, "X must be a 2-d [n, d] tensor");
  X = X.to(at::kFloat).contiguous();
  inscy_params p;
  p.neighborhood_size = (float)neighborhood_size;
  p.F = (float)F;
  p.num_obj = (int)num_obj;
  p.min_size = (int)min_size;
  p.r = (float)r;
  p.number_of_cells = (int)number_of_cells;
  p.rectangular = rectangular ? 1 : 0;
  p.entropy_order = (int)entropy_order;
  const int64_t n = X.size(0);
  const int d = (int)X.size(1);
  inscy_result* res = nullptr;
  int rc;
  if (X.is_cuda()) {
    const c10::cuda::CUDAGuard guard(X.device());
    void* stream = c10::cuda::getCurrentCUDAStream(X.device().index()).stream();
    rc = inscy_run_device(X.data_ptr<float>(), n, d, &p, mode, stream, &res);
  } else {
    rc = inscy_run(X.data_ptr<float>(), n, d, &p, mode, &res);
  }
  if (rc != INSCY_OK) throw std::runtime_error(std::string("inscy_gb300: ") + inscy_last_error());
  const int k = inscy_result_count(res);
  std::vector<std::vector<int>> subspaces(k), clusterings(k);
  int dims[64];
  for (int i = 0; i < k; ++i) {
    const int m = inscy_result_subspace(res, i, dims, 64);
    subspaces[i].assign(dims, dims + m);
    const int32_t* lab = inscy_result_labels_ptr(res, i);
    clusterings[i].assign(lab, lab + n);
  }
  inscy_result_free(res);
  return {subspaces, clusterings};
}

std::vector<std::vector<std::vector<int>>> run_gpu_5(at::Tensor X, double neighborhood_size, double F, int64_t num_obj,
                                                     int64_t min_size, double r, int64_t number_of_cells,
                                                     bool rectangular, int64_t entropy_order) {
  return run(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order,
             INSCY_MODE_BATCHED);
}

std::vector<std::vector<std::vector<int>>> run_gpu_4(at::Tensor X, double neighborhood_size, double F, int64_t num_obj,
                                                     int64_t min_size, double r, int64_t number_of_cells,
                                                     bool rectangular, int64_t entropy_order) {
  return run(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order,
             INSCY_MODE_PLAIN);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.doc() = "GB300 INSCY engine (libinscy_gb300.so) with the reference extension's entry points";
  m.def("run_gpu_5", &run_gpu_5, "INSCY, labels of the reference CPU INSCY (replaces inscy_map.cpp:1070 run_gpu_5)",
        py::arg("X"), py::arg("neighborhood_size"), py::arg("F"), py::arg("num_obj"), py::arg("min_size"),
        py::arg("r") = 1.0, py::arg("number_of_cells") = 3, py::arg("rectangular") = false,
        py::arg("entropy_order") = 0);
  m.def("run_gpu_4", &run_gpu_4, "INSCY, labels of the reference CPU INSCY (replaces inscy_map.cpp:979 run_gpu_4)",
        py::arg("X"), py::arg("neighborhood_size"), py::arg("F"), py::arg("num_obj"), py::arg("min_size"),
        py::arg("r") = 1.0, py::arg("number_of_cells") = 3, py::arg("rectangular") = false,
        py::arg("entropy_order") = 0);
  m.def("version", []() { return std::string(inscy_version()); });
}
