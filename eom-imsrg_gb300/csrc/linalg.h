// Small dense linear algebra on the host.
#pragma once
#include <vector>

namespace imsrg {

// Symmetric eigenproblem of a small n x n matrix (column-major): cyclic Jacobi.  Eigenvalues
// ascending in w, eigenvectors in the columns of V.
void jacobi_eigen(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V);

}  // namespace imsrg
