// Host-side set-up helpers of libtopopt_gb300 (no CUDA calls).
#pragma once
#include <cstdint>
#include <vector>

#include "tog_internal.h"

namespace tog {

template <int DIM>
struct ModalD {
    double D[1 << DIM][DIM];
    double O[1 << DIM][DIM][DIM];
};

void grid_counts(int dim, const int32_t* nel, long long* nnodes, long long* ncells);
void node_dofs_first_touch(int dim, const int32_t* nel, int32_t* node_dofs);
void cell_dofs_from_node_dofs(int dim, const int32_t* nel, const int32_t* node_dofs, int32_t* cell_dofs);
void element_stiffness(int dim, const double* size, double E, double nu, int plane_stress, double* Ke);
void modal_operator(int dim, const double* KeF, double* D_out, double* O_out, double* kd);
int filter_stencil(int dim, const double* size, double rmin, std::vector<int>& off, std::vector<double>& w);

}  // namespace tog
