/* Golden vectors of panopaea/src/dec/grid.rs (grid_2d_divergence :428-482,
 * grid_2d_laplacian :484-515), generated from grid_rs_vectors.json by
 * tests/golden/make_golden.py --header.  Do not edit. */
#pragma once
static const float GOLDEN_DIV_VELOCITIES_Y[30] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.8, 1.8, 0.0, 0.0, 0.0, 2.0, 2.0, 0.0, 0.0, 0.0, 0.8, 0.8, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
static const float GOLDEN_DIV_VELOCITIES_X[30] = {0.0, 0.7, 0.0, -0.7, 0.0, 0.0, 0.0, 0.1, 0.0, -0.1, 0.0, 0.0, 0.0, -0.7, 0.0, 0.7, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
static const float GOLDEN_DIV_REF[25] = {0.7, 1.1, 1.1, 0.7, 0.0, 0.1, 0.1, 0.1, 0.1, 0.0, -0.7, -0.5, -0.5, -0.7, 0.0, 0.0, -0.8, -0.8, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
static const double GOLDEN_DIV_EPS = 0.001;
static const double GOLDEN_LAP_FACES_PRIMAL[9] = {-0.0, -3.0, -0.0, -0.0, 2.0, 6.0, 1.0, -0.0, -0.0};
static const double GOLDEN_LAP_REF[9] = {3.0, -11.0, -3.0, -3.0, 5.0, 16.0, 2.0, -3.0, -6.0};
static const double GOLDEN_LAP_EPS = 0.001;
