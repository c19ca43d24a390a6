// Host eigendecomposition of a small dense symmetric FP64 matrix.
#pragma once

namespace sg {

// A: n x n column-major (only the lower triangle is read). On success w holds
// the eigenvalues in ascending order and V (n x n column-major) the matching
// orthonormal eigenvectors; returns 0, or 1 if the QL iteration did not
// converge within 60 sweeps of one eigenvalue.
int symeig_host(int n, const double* A, double* w, double* V);

}  // namespace sg
