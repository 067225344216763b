// Generated by tests/golden/make_cpp_goldens.py from reference_goldens.json;
// every value is cited there (test/testTensor.cu line ranges).
#pragma once
#include <vector>
namespace golden {
static const std::vector<double> addAB_a = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0, 13.0, 14.0, 15.0, 16.0, 17.0, 18.0};  // test/testTensor.cu:830-834 (tensorAddAB aData (2x3x3))
static const std::vector<double> addAB_b = {6.0, 5.0, 4.0, 3.0, 2.0, 1.0, 7.0, 6.0, 5.0, 4.0, 3.0, 2.0, 1.0, 2.0, 1.0, 5.0, -6.0, 8.0};  // test/testTensor.cu:835-839 (tensorAddAB bData (3x2x3))
static const std::vector<double> addAB_expected = {41.0, 56.0, 14.0, 20.0, 158.0, 176.0, 77.0, 86.0, 60.0, 64.0, 111.0, 118.0};  // test/testTensor.cu:844-844 (tensorAddAB expected C (2x2x3))
static const double chol_L00 = 3.16227766016838;  // test/testTensor.cu:1229
static const double chol_L21 = -0.361403161162101;  // test/testTensor.cu:1230
static const double chol_L22 = 5.382321781081287;  // test/testTensor.cu:1231
static const std::vector<double> chol_a = {10.0, 2.0, 3.0, 2.0, 20.0, -1.0, 3.0, -1.0, 30.0};  // test/testTensor.cu:1221-1225 (choleskyFactorisation aData (3x3))
static const std::vector<double> chol_b = {-1.0, -3.0, 5.0};  // test/testTensor.cu:1257-1257 (choleskyFactorisationSolution bData)
static const std::vector<double> chol_low_rowmajor = {3.16227766016838, 0.0, 0.0, 0.632455532033676, 4.427188724235731, 0.0, 0.948683298050514, -0.361403161162101, 5.382321781081287};  // test/testTensor.cu:1377-1381 (choleskyBatchSolve lowData (row-major L))
static const std::vector<double> chol_x = {-0.126805213103205, -0.128566396618528, 0.175061641423036};  // test/testTensor.cu:1262-1262 (choleskyFactorisationSolution expected x)
static const double dotF = 604.0;  // test/testTensor.cu:496
static const std::vector<double> getRows_a = {10.5, 25.0, 60.0, -21.0, 720.0, -1.0, 11.0, -1.0, 30.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0, 13.0};  // test/testTensor.cu:901-908 (tensorGetRows aData (3x3x2))
static const std::vector<double> getRows_expected0 = {25.0, 720.0, -1.0};  // test/testTensor.cu:911-911 (getRows(1,1,0))
static const std::vector<double> getRows_expected1 = {6.0, 7.0, 9.0, 10.0, 12.0, 13.0};  // test/testTensor.cu:917-917 (getRows(1,2,1))
static const double givens_a00 = 2.137186834969645;  // test/testTensor.cu:1726
static const double givens_a03 = 44.55212555975182;  // test/testTensor.cu:1727
static const double givens_a13 = -0.328797974610715;  // test/testTensor.cu:1728
static const std::vector<double> ls1_a = {1.0, 2.0, 3.0, 4.0, 7.0, 8.0, 9.0, 10.0, 6.0, 8.0, -9.0, 20.0};  // test/testTensor.cu:1015-1022 (tensorLeastSquares1 aData (2x2x3))
static const std::vector<double> ls1_b = {1.0, 1.0, -1.0, 2.0, 30.0, -80.0};  // test/testTensor.cu:1023-1023 (tensorLeastSquares1 bData (2x1x3))
static const double maxAbs = 27.0;  // test/testTensor.cu:551
static const double minAbs = 0.0;  // test/testTensor.cu:568
static const double normF = 26.153393661244042;  // test/testTensor.cu:517
static const std::vector<double> ns_a = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 7.0, 8.0, 9.0, 1.0, 2.0, 3.0, 4.0, 2.0, 4.0, 6.0, 8.0, 3.0, 6.0, 9.0, 12.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // test/testTensor.cu:1558-1564 (computeNullspaceTensor aData (3x4x5))
static const std::vector<double> ns_project_a_rowmajor = {1.0, -2.0, 3.0, 4.0, -1.0, -1.0, -1.0, 1.0, 2.0, -3.0, 4.0, -1.0, -1.0, -1.0, -1.0, 3.0, 5.0, -7.0, -1.0, -1.0, -1.0};  // test/testTensor.cu:1630-1634 (projectOnNullspaceTensor mat (3x7 row-major))
static const std::vector<double> ns_project_other = {1.0, -2.0, 5.0, 4.0, 0.0, 0.0, 0.0};  // test/testTensor.cu:1652-1652 (projectOnNullspaceTensor h_other)
static const std::vector<double> ns_project_x = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0};  // test/testTensor.cu:1641-1641 (projectOnNullspaceTensor vec)
static const std::vector<double> ns_trivial_rowmajor = {4.0, 5.0, 7.0, 4.0, 1.0, 8.0, 4.0, 5.0, 0.0, 1.0, 1.0, 1.0, 5.0, 6.0, 7.0, 9.0, 0.0, 3.0};  // test/testTensor.cu:1601-1608 (computeNullspaceTrivial data (3x3x2 row-major))
static const double precision_high = 1e-10;  // test/testTensor.cu:6
static const double precision_low = 0.0001;  // test/testTensor.cu:5
static const std::vector<double> qr_ls_a_rowmajor = {85.5638, -59.4001, -80.1992, 99.9464, 5.51393, 5.17935, 6.87488, -26.7536, 36.0914, -44.3857, -32.1268, 54.8915};  // test/testTensor.cu:1502-1507 (qrLeastSquares vecA (4x3 row-major))
static const std::vector<double> qr_ls_b = {-23.3585, -48.5744, 43.4229, -56.5081};  // test/testTensor.cu:1508-1513 (qrLeastSquares vecB)
static const double qr_ls_residual = 80.00316936419807;  // test/testTensor.cu:1529
static const double rank0 = 3.0;  // test/testTensor.cu:1191
static const double rank1 = 2.0;  // test/testTensor.cu:1192
static const double rank2 = 1.0;  // test/testTensor.cu:1193
static const std::vector<double> rank_a = {1.0, 4.0, 7.0, 10.0, 2.0, 5.0, 8.0, 11.0, 3.0, 6.0, 9.0, 0.0, 1.0, 4.0, 7.0, 10.0, 2.0, 5.0, 8.0, 11.0, 3.0, 6.0, 9.0, 12.0, 1.0, 2.0, 3.0, 4.0, 2.0, 4.0, 6.0, 8.0, 3.0, 6.0, 9.0, 12.0};  // test/testTensor.cu:1181-1185 (singularValuesRankMultipleMatrices aData (4x3x3))
static const double sumAbs = 112.0;  // test/testTensor.cu:534
static const std::vector<double> svd_b = {1.0, 6.0, 6.0, 6.0, 6.0, 6.0, 6.0, 6.0, 2.0, 7.0, 7.0, 7.0, 7.0, 7.0, 7.0, 7.0, 3.0, 8.0, 8.0, 8.0, 8.0, 8.0, 8.0, 8.0};  // test/testTensor.cu:1062-1066 (singularValuesComputation bData (8x3))
static const std::vector<double> svd_multi_a = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 1.0, 1.0, 1.0, 2.0, 2.0, 2.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0};  // test/testTensor.cu:1129-1129 (singularValuesMultipleMatrices aData (3x2x3))
static const std::vector<double> svd_multi_s = {9.508032000695726, 0.772869635673484, 3.872983346207417, 0.0, 1.0, 0.0};  // test/testTensor.cu:1146-1146 (expected_s)
static const std::vector<double> svd_multi_u = {-0.428667133548626, -0.566306918848035, -0.703946704147444, 0.805963908589298, 0.112382414096594, -0.58119908039611, 0.408248290463863, -0.816496580927726, 0.408248290463863, -0.577350269189626, -0.577350269189626, -0.577350269189626, 0.816496580927726, -0.408248290463863, -0.408248290463863, 0.0, -0.707106781186548, 0.707106781186547, 0.0, 0.0, -1.0, 1.0, 0.0, 0.0, 0.0, -1.0, 0.0};  // test/testTensor.cu:1151-1161 (expected_u (3x3x3))
static const std::vector<double> svd_multi_vt = {-0.386317703118612, -0.922365780077058, -0.922365780077058, 0.386317703118612, -0.447213595499958, -0.894427190999916, 0.894427190999916, -0.447213595499958, 0.0, -1.0, 1.0, 0.0};  // test/testTensor.cu:1137-1141 (expected_v (Vt, only first 4 checked))
static const double svd_sigma1 = 32.49624112375359;  // test/testTensor.cu:1074
static const double svd_sigma2 = 0.997152358903242;  // test/testTensor.cu:1075
static const std::vector<double> tensor_234A = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 8.0, 7.0, 10.0, 5.0, 4.0, 3.0, 2.0, 1.0, -1.0, 4.0, 3.0, 4.0, 3.0, 4.0, 8.0};  // test/testTensor.cu:21-21 (TENSOR_DATA_234A)
static const std::vector<double> tensor_234AMB = {-6.0, 8.0, -6.0, 2.0, 4.0, -5.0, -27.0, 9.0, 13.0, 11.0, -5.0, 3.0, -4.0, -5.0, 1.0, -7.0, 10.0, 2.0, 2.0, -2.0, 0.0, 8.0, 0.0, 3.0};  // test/testTensor.cu:24-24 (TENSOR_DATA_234AMB)
static const std::vector<double> tensor_234APB = {8.0, -4.0, 12.0, 6.0, 6.0, 17.0, 41.0, 7.0, 5.0, 5.0, 19.0, 17.0, 14.0, 13.0, 5.0, 11.0, -8.0, -4.0, 6.0, 8.0, 8.0, -2.0, 8.0, 13.0};  // test/testTensor.cu:23-23 (TENSOR_DATA_234APB)
static const std::vector<double> tensor_234B = {7.0, -6.0, 9.0, 2.0, 1.0, 11.0, 34.0, -1.0, -4.0, -3.0, 12.0, 7.0, 9.0, 9.0, 2.0, 9.0, -9.0, -3.0, 2.0, 5.0, 4.0, -5.0, 4.0, 5.0};  // test/testTensor.cu:22-22 (TENSOR_DATA_234B)
static const std::vector<double> transpose_a = {1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0};  // test/testTensor.cu:935-935 (tensorTranspose aData (3x2x2))
static const std::vector<double> transpose_expected = {1.0, 4.0, 2.0, 5.0, 3.0, 6.0, 7.0, 10.0, 8.0, 11.0, 9.0, 12.0};  // test/testTensor.cu:941-941 (tensorTranspose expected (2x3x2))
}  // namespace golden
