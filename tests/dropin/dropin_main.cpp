// Drop-in check: the reference's own training core (compiled from its sources) driven
// through CudaBackend. Without a GPU the backend must fail loudly with BackendError.
#include <cstdio>
#include <vector>

#include "mpsboost/trainer.hpp"
#include "mpsboost_cuda/cuda_backend.hpp"

int main() {
  using namespace mpsboost;
  std::vector<float> x(64 * 2);
  for (int i = 0; i < 128; ++i) x[i] = float(i);
  DenseMatrixView view{x.data(), 64, 2, 8, 4, ScalarType::kFloat32, true};
  BinnedDataset ds = QuantizeDense(view, 32);
  std::vector<double> y(64), w(64, 1.0);
  for (int i = 0; i < 64; ++i) y[i] = i < 32 ? -1.0 : 2.0;
  TrainingParameters p;
  p.n_estimators = 5;
  p.learning_rate = 0.3;
  p.max_bins = 32;
  p.tree.max_depth = 3;
  try {
    CudaBackend backend(0);
    RegressionModel model = TrainRegressionModel(ds, y, w, p, backend, backend);
    const std::vector<double> pred = model.Predict(ds);
    std::printf("trained %u trees, pred[0]=%.6f\n", model.tree_count(), pred[0]);
  } catch (const BackendError& e) {
    std::printf("BackendError: %s\n", e.what());
  }
  return 0;
}
