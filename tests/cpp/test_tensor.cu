// C++ acceptance tests of the drop-in tensor.cuh: the behaviour the
// reference's own test suite (test/testTensor.cu) checks, written against the
// same public API, for float and double (and int where the reference tests
// int).  Golden values come from goldens.h (read from the reference's tests).
// Prints one line per test and exits non-zero if any check failed.
#include <cstdio>
#include <random>
#include <functional>
#include <numeric>
#include <string>
#include <vector>

#include "tensor.cuh"
#include "goldens.h"

#define PRECISION_LOW 1e-4
#define PRECISION_HIGH 1e-10

// ------------------------------------------------------------ mini harness
static int g_fail_checks = 0;
static std::string g_current;
static bool g_test_failed = false;

static void report(bool ok, const char *expr, const char *file, int line) {
    if (ok) return;
    g_fail_checks++;
    g_test_failed = true;
    std::printf("  check failed in %s: %s (%s:%d)\n", g_current.c_str(), expr, file, line);
}

#define EXPECT_TRUE(c) report((c), #c, __FILE__, __LINE__)
#define EXPECT_EQ(a, b) report((a) == (b), #a " == " #b, __FILE__, __LINE__)
#define EXPECT_NE(a, b) report((a) != (b), #a " != " #b, __FILE__, __LINE__)
#define EXPECT_LT(a, b) report((a) < (b), #a " < " #b, __FILE__, __LINE__)
#define EXPECT_NEAR(a, b, tol) report(std::abs((double)(a) - (double)(b)) <= (tol), #a " ~ " #b, __FILE__, __LINE__)
#define EXPECT_THROW(stmt, exc)                         \
    do {                                                \
        bool thrown_ = false;                           \
        try { stmt; } catch (const exc &) { thrown_ = true; } \
        report(thrown_, #stmt " throws " #exc, __FILE__, __LINE__); \
    } while (0)

struct TestCase {
    std::string name;
    std::function<void()> fn;
};
static std::vector<TestCase> &registry() {
    static std::vector<TestCase> r;
    return r;
}
struct Registrar {
    Registrar(const char *n, std::function<void()> f) { registry().push_back({n, f}); }
};
#define TEST(name)                                    \
    static void name();                               \
    static Registrar reg_##name(#name, name);         \
    static void name()

template <typename T>
static std::vector<T> as(const std::vector<double> &v) {
    return std::vector<T>(v.begin(), v.end());
}

// ------------------------------------------------------------- DTensor
template <typename T> static void constructionZero() {
    DTensor<T> zero(2, 3, 4, true);
    EXPECT_EQ(2u, zero.numRows()); EXPECT_EQ(3u, zero.numCols()); EXPECT_EQ(4u, zero.numMats());
    std::vector<T> down;
    zero.download(down);
    EXPECT_TRUE(down == std::vector<T>(24, 0));
}
TEST(tensorConstructionZero) { constructionZero<float>(); constructionZero<double>(); constructionZero<int>(); }

template <typename T> static void storageMode() {
    const std::vector<T> cm = {1, 3, 5, 2, 4, 6, 7, 9, 11, 8, 10, 12};
    const std::vector<T> rm = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
    std::vector<T> host;
    DTensor<T> a(cm, 3, 2, 2, columnMajor), b(rm, 3, 2, 2, rowMajor);
    a.download(host); EXPECT_TRUE(host == cm);
    b.download(host); EXPECT_TRUE(host == cm);
    DTensor<T> split(3, 2, 2);
    DTensor<T> s0(split, 2, 0, 0), s1(split, 2, 1, 1);
    s0.upload({1, 2, 3, 4, 5, 6}, rowMajor);
    s1.upload({7, 8, 9, 10, 11, 12}, rowMajor);
    split.download(host); EXPECT_TRUE(host == cm);
}
TEST(tensorConstructionStorageMode) { storageMode<float>(); storageMode<double>(); storageMode<int>(); }

template <typename T> static void randomTensor() {
    auto r = DTensor<T>::createRandomTensor(20, 40, 60, -1, 1);
    EXPECT_EQ(60u, r.numMats());
    T e = r(19, 39, 59);
    EXPECT_TRUE(e >= -1 && e <= 1);
}
TEST(randomTensorCreation) { randomTensor<float>(); randomTensor<double>(); randomTensor<int>(); }

template <typename T> static void fileRoundTrip(const std::string &fname) {
    auto r = DTensor<T>::createRandomTensor(20, 40, 6, -1, 1);
    r.saveToFile(fname);
    auto a = DTensor<T>::parseFromFile(fname);
    EXPECT_EQ(20u, a.numRows()); EXPECT_EQ(40u, a.numCols()); EXPECT_EQ(6u, a.numMats());
    auto diff = a - r;
    EXPECT_LT(diff.maxAbs(), 2 * std::numeric_limits<T>::epsilon());
}
TEST(parseTensorFromFile) { fileRoundTrip<float>("_dropin_test.dtensor"); fileRoundTrip<double>("_dropin_test.dtensor"); }
TEST(parseTensorFromFileBinary) { fileRoundTrip<float>("_dropin_test.bt"); fileRoundTrip<double>("_dropin_test.bt"); }

TEST(parseTensorFromBinaryPython) {
    // written by the reference's python API (python/test/test.py:9-13)
    auto b = DTensor<double>::parseFromFile(std::string(GOLDEN_DIR) + "/b_d.bt");
    for (size_t i = 0; i < 3; i++)
        for (size_t j = 0; j < 3 && j < b.numCols(); j++) {
            EXPECT_NEAR(1 + 2 * j + 6 * i, b(i, j, 0), PRECISION_HIGH);
            EXPECT_NEAR(2 + 2 * j + 6 * i, b(i, j, 1), PRECISION_HIGH);
        }
}

TEST(parseTensorFromNonexistentFile) {
    EXPECT_THROW(DTensor<double>::parseFromFile("_no_such_file.bt", rowMajor), std::invalid_argument);
    EXPECT_THROW(DTensor<double>::parseFromFile("_no_such_file.txt", rowMajor), std::invalid_argument);
}

template <typename T> static void moveConstruct() {
    DTensor<T> zero(2, 3, 4, true);
    DTensor<T> x(std::move(zero));
    EXPECT_EQ(0u, zero.numEl());
    EXPECT_EQ(24u, x.numEl());
    DTensor<T> y(DTensor<T>{100, 10, 1000});
    EXPECT_EQ(1000000u, y.numEl());
}
TEST(tensorMoveConstructor) { moveConstruct<float>(); moveConstruct<double>(); moveConstruct<int>(); }

template <typename T> static void copyConstruct() {
    auto data = as<T>(golden::tensor_234A);
    DTensor<T> t(data, 2, 3, 4);
    DTensor<T> c(t);
    std::vector<T> down;
    c.download(down);
    EXPECT_TRUE(down == data);
    EXPECT_NE(t.raw(), c.raw());
    EXPECT_EQ(24u, c.numEl());
}
TEST(tensorCopyConstructor) { copyConstruct<float>(); copyConstruct<double>(); copyConstruct<int>(); }

template <typename T> static void slicing() {
    DTensor<T> t(as<T>(golden::tensor_234A), 2, 3, 4);
    DTensor<T> s2(t, 2, 0, 1);
    EXPECT_EQ(2u, s2.numMats()); EXPECT_EQ(t.raw(), s2.raw()); EXPECT_TRUE(s2.ptrMatrices() != nullptr);
    DTensor<T> s1(t, 1, 1, 2);
    EXPECT_EQ(2u, s1.numCols()); EXPECT_TRUE(s1.ptrMatrices() == nullptr);
    std::vector<T> d;
    s1.download(d); EXPECT_TRUE(d == std::vector<T>({3, 4, 5, 6}));
    DTensor<T> s0(t, 0, 2, 3);
    s0.download(d); EXPECT_TRUE(d == std::vector<T>({3, 4}));
    DTensor<T> s3(t, 2, 2, 3);
    EXPECT_TRUE(s3.ptrMatrices() == t.ptrMatrices() + 2);
}
TEST(tensorSlicing) { slicing<float>(); slicing<double>(); slicing<int>(); }

template <typename T> static void uploadAndBracket() {
    DTensor<T> t(2, 3, 4);
    t.upload(as<T>(golden::tensor_234A));
    EXPECT_EQ(T(8), t(1, 2, 3));
    EXPECT_EQ(T(1), t(0, 0, 0));
    EXPECT_EQ(T(3), t(0, 1, 2));
}
TEST(tensorUploadAndBracket) { uploadAndBracket<float>(); uploadAndBracket<double>(); uploadAndBracket<int>(); }

template <typename T> static void deviceCopy() {
    DTensor<T> t(as<T>(golden::tensor_234A), 2, 3, 4);
    DTensor<T> other(2, 3, 5, true);
    DTensor<T> z(other, 2, 1, 4);
    t.deviceCopyTo(z);
    std::vector<T> expect(6, 0);
    auto a = as<T>(golden::tensor_234A);
    expect.insert(expect.end(), a.begin(), a.end());
    std::vector<T> got;
    other.download(got);
    EXPECT_TRUE(got == expect);
}
TEST(tensorDeviceCopyTo) { deviceCopy<float>(); deviceCopy<double>(); deviceCopy<int>(); }

template <typename T> static void reshape() {
    size_t m = 5, n = 10, k = 3;
    auto a = DTensor<T>::createRandomTensor(m, n, k, -1, 1);
    T last = a(m - 1, n - 1, k - 1), first = a(0, 0, 0);
    a.reshape(m, k, n); EXPECT_EQ(n, a.numMats());
    a.reshape(k, n, m); EXPECT_EQ(m, a.numMats());
    a.reshape(k * n, m, 1); EXPECT_EQ(1u, a.numMats());
    a.reshape(m * k * n, 1, 1);
    EXPECT_EQ(last, a(m * n * k - 1, 0, 0));
    EXPECT_EQ(first, a(0, 0, 0));
    EXPECT_THROW(a.reshape(7, 7, 7), std::invalid_argument);
}
TEST(tensorReshape) { reshape<float>(); reshape<double>(); reshape<int>(); }

template <typename T> static void sliceReshapeAdd(T eps) {
    DTensor<T> a(as<T>(golden::tensor_234A), 2, 3, 4), b(as<T>(golden::tensor_234B), 2, 3, 4);
    DTensor<T> as_(a, 2, 1, 3), bs(b, 2, 1, 3);
    as_.reshape(2, 9, 1);
    bs.reshape(2, 9, 1);
    as_ += bs;
    std::vector<T> expect = {1, 2, 3, 4, 5, 6, 41, 7, 5, 5, 19, 17, 14, 13, 5, 11, -8, -4, 6, 8, 8, -2, 8, 13};
    DTensor<T> e(expect, 2, 3, 4);
    DTensor<T> err = e - a;
    EXPECT_LT(err.normF(), eps);
}
TEST(tensorSliceAndReshape) { sliceReshapeAdd<float>(PRECISION_LOW); sliceReshapeAdd<double>(PRECISION_HIGH); }

template <typename T> static void reductions(T eps) {
    auto A = as<T>(golden::tensor_234A), B = as<T>(golden::tensor_234B);
    DTensor<T> va(A, A.size()), vb(B, B.size());
    EXPECT_EQ(T(golden::dotF), va.dotF(vb));
    DTensor<T> ta(A, 2, 3, 4), tb(B, 2, 3, 4);
    EXPECT_EQ(T(golden::dotF), ta.dotF(tb));
    EXPECT_NEAR(golden::normF, ta.normF(), eps);
    EXPECT_NEAR(golden::sumAbs, ta.sumAbs(), PRECISION_HIGH);
    DTensor<T> amb(as<T>(golden::tensor_234AMB), 2, 3, 4);
    EXPECT_EQ(T(golden::maxAbs), amb.maxAbs());
    EXPECT_EQ(T(golden::minAbs), amb.minAbs());
}
TEST(tensorReductions) { reductions<float>(PRECISION_LOW); reductions<double>(PRECISION_HIGH); }

template <typename T> static void rightGivens(T eps) {
    size_t m = 10, n = 6;
    std::vector<T> v(m * n);
    std::iota(v.begin(), v.end(), T(1));
    DTensor<T> a(v, m, n, 1);
    T c = 0.1, minus_s = std::sqrt(1 - c * c);
    a.applyRightGivensRotation(1, 4, &c, &minus_s);
    for (size_t i = 0; i < m; i++) {
        EXPECT_NEAR(1 + i, a(i, 0), eps);
        EXPECT_NEAR(21 + i, a(i, 2), eps);
        EXPECT_NEAR((11 + i) * c - (41 + i) * (-minus_s), a(i, 1), eps);
        EXPECT_NEAR((11 + i) * (-minus_s) + (41 + i) * c, a(i, 4), eps);
    }
}
TEST(tensorRightGivens) { rightGivens<float>(PRECISION_LOW); rightGivens<double>(PRECISION_HIGH); }

TEST(tensorLeftGivens) {
    size_t m = 10, n = 6;
    std::vector<double> v(m * n);
    std::iota(v.begin(), v.end(), 1.0);
    DTensor<double> a(v, m, n, 1);
    double c = 0.1, minus_s = -std::sqrt(1 - c * c);
    a.applyLeftGivensRotation(1, 9, &c, &minus_s);
    for (size_t j = 0; j < n; j++) {
        EXPECT_NEAR(1 + 10 * j, a(0, j), 1e-14);
        for (size_t i = 2; i < m - 1; i++) EXPECT_NEAR(1 + i + 10 * j, a(i, j), 1e-14);
        EXPECT_NEAR((2 + 10 * j) * c + (10 + 10 * j) * minus_s, a(1, j), 1e-12);
        EXPECT_NEAR((2 + 10 * j) * (-minus_s) + (10 + 10 * j) * c, a(9, j), 1e-12);
    }
}

template <typename T> static void assignAndArith() {
    DTensor<T> t(as<T>(golden::tensor_234A), 2, 3, 4);
    DTensor<T> other;
    other = t;
    EXPECT_EQ(t.raw(), other.raw());
    EXPECT_EQ(4u, other.numMats());
    std::vector<T> three;
    for (double x : golden::tensor_234A) three.push_back(T(3 * x));
    DTensor<T> u(as<T>(golden::tensor_234A), 2, 3, 4);
    u *= 3.0;
    std::vector<T> d;
    u.download(d); EXPECT_TRUE(d == three);
    DTensor<T> w(as<T>(golden::tensor_234A), 2, 3, 4);
    auto tri = T(3) * w;
    tri.download(d); EXPECT_TRUE(d == three);
    DTensor<T> A(as<T>(golden::tensor_234A), 2, 3, 4), B(as<T>(golden::tensor_234B), 2, 3, 4);
    DTensor<T> P = A + B, M = A - B;
    P.download(d); EXPECT_TRUE(d == as<T>(golden::tensor_234APB));
    M.download(d); EXPECT_TRUE(d == as<T>(golden::tensor_234AMB));
    A += B;
    A.download(d); EXPECT_TRUE(d == as<T>(golden::tensor_234APB));
    A -= B; A -= B;
    A.download(d); EXPECT_TRUE(d == as<T>(golden::tensor_234AMB));
}
TEST(tensorAssignmentAndArithmetic) { assignAndArith<float>(); assignAndArith<double>(); }

template <typename T> static void addAB() {
    DTensor<T> A(as<T>(golden::addAB_a), 2, 3, 3), B(as<T>(golden::addAB_b), 3, 2, 3);
    DTensor<T> C(2, 2, 3, true);
    C.addAB(A, B);
    std::vector<T> d;
    C.download(d);
    EXPECT_TRUE(d == as<T>(golden::addAB_expected));
    DTensor<T> bad(3, 3, 3);
    EXPECT_THROW(C.addAB(A, bad), std::invalid_argument);
}
TEST(tensorAddAB) { addAB<double>(); addAB<float>(); }

template <typename T> static void getRowsTr() {
    DTensor<T> A(as<T>(golden::getRows_a), 3, 3, 2);
    std::vector<T> d;
    A.getRows(1, 1, 0).download(d); EXPECT_TRUE(d == as<T>(golden::getRows_expected0));
    A.getRows(1, 2, 1).download(d); EXPECT_TRUE(d == as<T>(golden::getRows_expected1));
    DTensor<T> X(as<T>(golden::transpose_a), 3, 2, 2);
    DTensor<T> Xt = X.tr();
    EXPECT_EQ(2u, Xt.numRows()); EXPECT_EQ(3u, Xt.numCols()); EXPECT_EQ(2u, Xt.numMats());
    Xt.download(d); EXPECT_TRUE(d == as<T>(golden::transpose_expected));
}
TEST(tensorGetRowsAndTranspose) { getRowsTr<float>(); getRowsTr<double>(); }

template <typename T> static void bytesAllocated() {
    size_t before = Session::getInstance().totalAllocatedBytes();
    size_t m = 10, n = 10, k = 20;
    auto *A = new DTensor<T>(m, n, k);
    EXPECT_EQ(before + m * n * k * sizeof(T) + k * sizeof(T *), Session::getInstance().totalAllocatedBytes());
    delete A;
    EXPECT_EQ(before, Session::getInstance().totalAllocatedBytes());
}
TEST(tensorBytesAllocated) { bytesAllocated<float>(); bytesAllocated<double>(); bytesAllocated<int>(); }

// ------------------------------------------------------------ least squares
template <typename T> static void leastSquares1(T eps) {
    DTensor<T> A0(as<T>(golden::ls1_a), 2, 2, 3);
    DTensor<T> A(A0);
    DTensor<T> B(as<T>(golden::ls1_b), 2, 1, 3);
    DTensor<T> sol(B);
    A0.leastSquaresBatched(sol);
    DTensor<T> C(2, 1, 3);
    C.addAB(A, sol);
    C -= B;
    EXPECT_LT(C.normF(), eps);
}
TEST(tensorLS1) { leastSquares1<float>(PRECISION_LOW); leastSquares1<double>(PRECISION_HIGH); }

// ---------------------------------------------------------------------- SVD
template <typename T> static void svdValues(T eps) {
    DTensor<T> B(as<T>(golden::svd_b), 8, 3);
    Svd<T> svd(B, true, false);
    svd.factorise();
    EXPECT_EQ(0, svd.info()(0));
    auto S = svd.singularValues();
    EXPECT_NEAR(golden::svd_sigma1, S(0), eps);
    EXPECT_NEAR(golden::svd_sigma2, S(1), eps);
    EXPECT_TRUE(svd.leftSingularVectors().has_value());
    // memory: the same objects every call
    EXPECT_EQ(&svd.rightSingularVectors(), &svd.rightSingularVectors());
    EXPECT_EQ(&svd.singularValues(), &svd.singularValues());
    EXPECT_EQ(svd.leftSingularVectors().value(), svd.leftSingularVectors().value());
}
TEST(singularValuesComputationAndMemory) { svdValues<float>(PRECISION_LOW); svdValues<double>(PRECISION_HIGH); }

template <typename T> static void svdMultiple(T eps) {
    DTensor<T> A(as<T>(golden::svd_multi_a), 3, 2, 3);
    Svd<T> svd(A, true);
    svd.factorise();
    std::vector<T> v, s, u;
    svd.rightSingularVectors().download(v);
    svd.singularValues().download(s);
    svd.leftSingularVectors().value()->download(u);
    for (size_t i = 0; i < 4; i++) EXPECT_NEAR(golden::svd_multi_vt[i], v[i], eps);
    for (size_t i = 0; i < 6; i++) EXPECT_NEAR(golden::svd_multi_s[i], s[i], eps);
    for (size_t i = 0; i < 27; i++) EXPECT_NEAR(golden::svd_multi_u[i], u[i], eps);
}
TEST(singularValuesMultipleMatrices) { svdMultiple<float>(10 * PRECISION_LOW); svdMultiple<double>(PRECISION_HIGH); }

template <typename T> static void svdRank(T eps) {
    DTensor<T> A(as<T>(golden::rank_a), 4, 3, 3);
    Svd<T> svd(A);
    svd.factorise();
    auto rank = svd.rank(eps);
    EXPECT_EQ((unsigned)golden::rank0, rank(0, 0, 0));
    EXPECT_EQ((unsigned)golden::rank1, rank(0, 0, 1));
    EXPECT_EQ((unsigned)golden::rank2, rank(0, 0, 2));
    auto again = svd.rank(eps);  // written, not accumulated
    EXPECT_EQ((unsigned)golden::rank0, again(0, 0, 0));
    DTensor<T> fat(2, 3, 1);
    EXPECT_THROW(Svd<T>{fat}, std::invalid_argument);
}
TEST(singularValuesRankMultipleMatrices) { svdRank<float>(PRECISION_LOW); svdRank<double>(PRECISION_HIGH); }

// ----------------------------------------------------------------- Cholesky
template <typename T> static void cholesky(T eps) {
    auto a = as<T>(golden::chol_a);
    DTensor<T> A(a, 3, 3, 1);
    CholeskyFactoriser<T> chol(A);
    chol.factorise();
    EXPECT_NEAR(golden::chol_L00, A(0, 0), eps);
    EXPECT_NEAR(golden::chol_L21, A(2, 1), eps);
    EXPECT_NEAR(golden::chol_L22, A(2, 2), eps);
    EXPECT_EQ(0, chol.info()(0));
    DTensor<T> A2(a, 3, 3, 1), L(A2);
    CholeskyFactoriser<T> c2(L);
    c2.factorise();
    DTensor<T> rhs(as<T>(golden::chol_b), 3, 1, 1), sol(rhs);
    c2.solve(sol);
    std::vector<T> x;
    sol.download(x);
    for (int i = 0; i < 3; i++) EXPECT_NEAR(golden::chol_x[i], x[i], eps);
    DTensor<T> err = A2 * sol;
    err -= rhs;
    EXPECT_LT(err.normF(), eps);
    DTensor<T> rect(3, 2, 1);
    EXPECT_THROW(CholeskyFactoriser<T>{rect}, std::invalid_argument);
}
TEST(choleskyFactorisationAndSolution) { cholesky<float>(PRECISION_LOW); cholesky<double>(PRECISION_HIGH); }

template <typename T> static void choleskyBatch(T eps) {
    auto a = as<T>(golden::chol_a);
    DTensor<T> A(3, 3, 2);
    DTensor<T> A0(A, 2, 0, 0), A1(A, 2, 1, 1);
    A0.upload(a); A1.upload(a);
    DTensor<T> L(A);
    CholeskyBatchFactoriser<T> chol(L);
    DTensor<T> early(3, 1, 2);
    EXPECT_THROW(chol.solve(early), std::logic_error);
    chol.factorise();
    for (size_t k = 0; k < 2; k++) {
        EXPECT_NEAR(golden::chol_L00, L(0, 0, k), eps);
        EXPECT_NEAR(golden::chol_L21, L(2, 1, k), eps);
        EXPECT_NEAR(golden::chol_L22, L(2, 2, k), eps);
    }
    DTensor<T> rhs(3, 1, 2);
    DTensor<T> r0(rhs, 2, 0, 0), r1(rhs, 2, 1, 1);
    r0.upload(as<T>(golden::chol_b)); r1.upload(as<T>(golden::chol_b));
    DTensor<T> sol(rhs);
    chol.solve(sol);
    std::vector<T> x;
    sol.download(x);
    for (int i = 0; i < 3; i++) { EXPECT_NEAR(golden::chol_x[i], x[i], eps); EXPECT_NEAR(golden::chol_x[i], x[i + 3], eps); }
    DTensor<T> err = A * sol;
    err -= rhs;
    EXPECT_LT(err.normF(), eps);
    EXPECT_EQ(0, chol.info()(0));
    // pre-factored L (factorised = true)
    DTensor<T> low(3, 3, 2);
    DTensor<T> l0(low, 2, 0, 0), l1(low, 2, 1, 1);
    l0.upload(as<T>(golden::chol_low_rowmajor), rowMajor);
    l1.upload(as<T>(golden::chol_low_rowmajor), rowMajor);
    CholeskyBatchFactoriser<T> pre(low, true);
    DTensor<T> sol2(rhs);
    pre.solve(sol2);
    sol2.download(x);
    for (int i = 0; i < 3; i++) EXPECT_NEAR(golden::chol_x[i], x[i + 3], eps);
}
TEST(choleskyBatchFactorisationAndSolve) { choleskyBatch<float>(PRECISION_LOW); choleskyBatch<double>(PRECISION_HIGH); }

// ----------------------------------------------------------------------- QR
template <typename T> static void qrFactor(size_t nR, size_t nC, T eps) {
    DTensor<T> temp(nR, nC);
    auto A = DTensor<T>::createRandomTensor(nR, nC, 1, -100, 100);
    QRFactoriser<T> qr(temp);
    A.deviceCopyTo(temp);
    qr.factorise();
    EXPECT_EQ(0, qr.info()(0));
    DTensor<T> Q(nR, nC), R(nC, nC, 1, true), QR(nR, nC);
    qr.getQR(Q, R);
    QR.addAB(Q, R);
    QR -= A;
    EXPECT_NEAR(QR.normF(), 0., eps * 100);  // entries up to 100 (the reference's tolerance is absolute)
}
TEST(qrFactorisation) {
    qrFactor<float>(4, 3, PRECISION_LOW); qrFactor<double>(4, 3, PRECISION_HIGH);
    qrFactor<float>(20, 3, PRECISION_LOW); qrFactor<double>(20, 3, PRECISION_HIGH);
}

template <typename T> static void qrLS(T eps) {
    size_t nR = 4, nC = 3;
    DTensor<T> temp(nR, nC);
    DTensor<T> A(as<T>(golden::qr_ls_a_rowmajor), nR, nC, 1, rowMajor);
    DTensor<T> b(as<T>(golden::qr_ls_b), nR);
    DTensor<T> xFull(nR);
    DTensor<T> x(xFull, 0, 0, nC - 1);
    DTensor<T> Ax(nR);
    QRFactoriser<T> qr(temp);
    A.deviceCopyTo(temp);
    qr.factorise();
    b.deviceCopyTo(xFull);
    qr.leastSquares(xFull);
    EXPECT_EQ(0, qr.info()(0));
    Ax.addAB(A, x);
    Ax -= b;
    EXPECT_NEAR(Ax.normF(), golden::qr_ls_residual, eps);
}
TEST(qrLeastSquares) { qrLS<float>(PRECISION_LOW); qrLS<double>(PRECISION_HIGH); }

// ---------------------------------------------------------------- Nullspace
template <typename T> static void nullspaceTensor(T eps) {
    DTensor<T> A(as<T>(golden::ns_a), 3, 4, 5);
    Nullspace<T> ns(A);
    DTensor<T> nA = ns.nullspace();
    EXPECT_EQ(5u, nA.numMats());
    for (size_t i = 0; i < 5; i++) {
        DTensor<T> nAi(nA, 2, i, i), Ai(A, 2, i, i);
        DTensor<T> zero = Ai * nAi;
        EXPECT_LT(zero.normF(), eps);
        DTensor<T> nAiTr = nAi.tr();
        DTensor<T> eye = nAiTr * nAi;
        EXPECT_NEAR(1, eye(0, 0, 0), eps);
        for (size_t r = 0; r < eye.numRows(); r++)
            for (size_t c = 0; c < eye.numCols(); c++)
                if (r != c) EXPECT_NEAR(0, eye(r, c, 0), eps);
    }
}
TEST(computeNullspaceTensor) { nullspaceTensor<float>(PRECISION_LOW); nullspaceTensor<double>(PRECISION_HIGH); }

template <typename T> static void nullspaceTrivial() {
    DTensor<T> A(as<T>(golden::ns_trivial_rowmajor), 3, 3, 2, rowMajor);
    Nullspace<T> ns(A);
    DTensor<T> N = ns.nullspace();
    EXPECT_EQ(T(0), N.normF());
}
TEST(computeNullspaceTrivial) { nullspaceTrivial<float>(); nullspaceTrivial<double>(); }

template <typename T> static void nullspaceProject(T eps) {
    size_t m = 3, n = 7;
    DTensor<T> A(m, n, 1);
    A.upload(as<T>(golden::ns_project_a_rowmajor), rowMajor);
    Nullspace<T> ns(A);
    DTensor<T> N = ns.nullspace();
    DTensor<T> x(as<T>(golden::ns_project_x), n);
    DTensor<T> proj(x);
    ns.project(proj);
    DTensor<T> error(m, 1, 1, true);
    error.addAB(A, proj);
    EXPECT_LT(error.normF(), eps);
    DTensor<T> other(as<T>(golden::ns_project_other), n);
    DTensor<T> y = N * other;
    DTensor<T> d1 = y - proj, d2 = proj - x;
    EXPECT_LT(d1.dotF(d2), eps);
    DTensor<T> tall(4, 3, 1);
    EXPECT_THROW(Nullspace<T>{tall}, std::invalid_argument);
}
TEST(projectOnNullspaceTensor) { nullspaceProject<float>(PRECISION_LOW); nullspaceProject<double>(PRECISION_HIGH); }

// -------------------------------------------------------- GivensAnnihilator
template <typename T> static void givensAnnihilate(T eps) {
    size_t m = 10, n = 6;
    std::vector<T> v(m * n);
    std::iota(v.begin(), v.end(), T(1));
    DTensor<T> a(v, m, n, 1);
    GivensAnnihilator<T> ga(a);
    for (size_t k = 1; k < m; k++)
        for (size_t j = 0; j < n; j++) {
            ga.annihilate(0, k, j);
            EXPECT_NEAR(0.0, a(k, j), eps * 10);
        }
    EXPECT_THROW(ga.annihilate(0, m, 0), std::invalid_argument);
    EXPECT_THROW(ga.annihilate(0, 1, n), std::invalid_argument);
}
TEST(givensAnnihilateElement) { givensAnnihilate<float>(PRECISION_LOW); givensAnnihilate<double>(PRECISION_HIGH); }

TEST(givensAnnihilateCorrectness) {
    size_t m = 10, n = 6;
    std::vector<double> v(m * n);
    std::iota(v.begin(), v.end(), 1.0);
    DTensor<double> a(v, m, n);
    GivensAnnihilator<double> ga(a);
    ga.annihilate(0, 1, 2);
    EXPECT_NEAR(0.0, a(1, 2), 1e-14);
    EXPECT_NEAR(golden::givens_a00, a(0, 0), 1e-12);
    EXPECT_NEAR(golden::givens_a03, a(0, 3), 1e-12);
    EXPECT_NEAR(golden::givens_a13, a(1, 3), 1e-12);
}

// ------------------------------------- shapes beyond the warp kernels (extensions of coverage)
template <typename T> static std::vector<T> randomVec(size_t len, unsigned seed) {
    std::mt19937 gen(seed);
    std::normal_distribution<double> d(0.0, 1.0);
    std::vector<T> v(len);
    for (auto &x : v) x = (T)d(gen);
    return v;
}

// leastSquaresBatched on 128 x 64 (and 100 x 50): the normal equations hold
template <typename T> static void lsBig(size_t m, size_t n, T eps) {
    const size_t k = 3;
    std::vector<T> a = randomVec<T>(m * n * k, 11), b = randomVec<T>(m * k, 12);
    DTensor<T> A(a, m, n, k), B(b, m, 1, k), A0(a, m, n, k), B0(b, m, 1, k);
    A.leastSquaresBatched(B);
    std::vector<T> x;
    B.download(x);
    for (size_t i = 0; i < k; i++) {
        // A^T (b - A x) = 0 relative to |A| |b|
        double worst = 0, na = 0, nb = 0;
        for (size_t e = 0; e < m * n; e++) na += (double)a[i * m * n + e] * a[i * m * n + e];
        for (size_t r = 0; r < m; r++) nb += (double)b[i * m + r] * b[i * m + r];
        std::vector<double> res(m);
        for (size_t r = 0; r < m; r++) {
            double acc = b[i * m + r];
            for (size_t c = 0; c < n; c++) acc -= (double)a[i * m * n + c * m + r] * x[i * m + c];
            res[r] = acc;
        }
        for (size_t c = 0; c < n; c++) {
            double g = 0;
            for (size_t r = 0; r < m; r++) g += (double)a[i * m * n + c * m + r] * res[r];
            worst = std::max(worst, std::abs(g));
        }
        EXPECT_LT(worst / std::sqrt(na * nb), eps);
    }
}
TEST(leastSquaresBatchedBeyond128x32) {
    lsBig<float>(128, 64, 1e-5f); lsBig<double>(128, 64, 1e-12);
    lsBig<float>(100, 50, 1e-5f); lsBig<double>(256, 100, 1e-12);
}

// QRFactoriser on 100 x 50: Q R == A, Q^T Q == I, least squares as above
template <typename T> static void qrBig(size_t m, size_t n, T eps) {
    std::vector<T> a = randomVec<T>(m * n, 21);
    DTensor<T> A(a, m, n), work(a, m, n);
    QRFactoriser<T> qr(work);
    qr.factorise();
    EXPECT_EQ(0, qr.info()(0));
    DTensor<T> Q(m, n), R(n, n);
    qr.getQR(Q, R);
    DTensor<T> QR_(m, n);
    QR_.addAB(Q, R);
    QR_ -= A;
    EXPECT_LT(QR_.normF() / A.normF(), eps);
    DTensor<T> QtQ(n, n);
    DTensor<T> Qt = Q.tr();
    QtQ.addAB(Qt, Q);
    std::vector<T> q;
    QtQ.download(q);
    double worst = 0;
    for (size_t c = 0; c < n; c++)
        for (size_t r = 0; r < n; r++) worst = std::max(worst, std::abs((double)q[c * n + r] - (r == c ? 1.0 : 0.0)));
    EXPECT_LT(worst, eps * 10);
}
TEST(qrFactoriserBeyond128x32) { qrBig<float>(100, 50, 1e-5f); qrBig<double>(256, 100, 1e-12); qrBig<double>(128, 128, 1e-12); }

// Svd with U on 96 x 96 and 200 x 128: A == U S V^T, S descending
template <typename T> static void svdBig(size_t m, size_t n, T eps) {
    std::vector<T> a = randomVec<T>(m * n, 31);
    DTensor<T> A(a, m, n);
    Svd<T> svd(A, true, false);
    svd.factorise();
    EXPECT_EQ(0, svd.info()(0));
    std::vector<T> S, Vt, U;
    svd.singularValues().download(S);
    svd.rightSingularVectors().download(Vt);
    (*svd.leftSingularVectors().value()).download(U);
    for (size_t j = 1; j < n; j++) EXPECT_TRUE(S[j] <= S[j - 1]);
    double num = 0, den = 0;
    for (size_t c = 0; c < n; c++)
        for (size_t r = 0; r < m; r++) {
            double acc = 0;
            for (size_t l = 0; l < n; l++) acc += (double)U[l * m + r] * S[l] * Vt[c * n + l];
            num += (acc - a[c * m + r]) * (acc - a[c * m + r]);
            den += (double)a[c * m + r] * a[c * m + r];
        }
    EXPECT_LT(std::sqrt(num / den), eps);
}
TEST(svdBeyond64Columns) { svdBig<float>(96, 96, 1e-5f); svdBig<float>(200, 128, 1e-5f); svdBig<double>(128, 128, 1e-12); }

// Nullspace of 100 x 140: A N == 0, N^T N == I on the kernel columns
template <typename T> static void nullspaceBig(size_t m, size_t n, T eps) {
    std::vector<T> a = randomVec<T>(m * n, 41);
    DTensor<T> A(a, m, n);
    Nullspace<T> ns(A);
    DTensor<T> N = ns.nullspace();
    DTensor<T> AN(m, n);
    AN.addAB(A, N);
    EXPECT_LT(AN.normF(), eps * A.normF());
    DTensor<T> Nt = N.tr();
    DTensor<T> NtN(n, n);
    NtN.addAB(Nt, N);
    std::vector<T> g;
    NtN.download(g);
    double tr = 0;
    for (size_t i = 0; i < n; i++) tr += g[i * n + i];
    EXPECT_NEAR(tr, (double)(n - m), 1e-3);
}
TEST(nullspaceBeyond64Rows) { nullspaceBig<float>(100, 140, 1e-4f); nullspaceBig<double>(120, 130, 1e-10); }

// CholeskyBatchFactoriser for n = 200 (shared memory, float) and 300 (global memory, double)
template <typename T> static void choleskyBig(size_t n, T eps) {
    const size_t k = 2;
    std::vector<T> g = randomVec<T>(n * n * k, 51), a(n * n * k, T(0));
    for (size_t i = 0; i < k; i++)
        for (size_t c = 0; c < n; c++)
            for (size_t r = 0; r < n; r++) {
                double acc = r == c ? 0.5 : 0.0;
                for (size_t l = 0; l < n; l++) acc += (double)g[i * n * n + r * n + l] * g[i * n * n + c * n + l] / n;
                a[i * n * n + c * n + r] = (T)acc;
            }
    DTensor<T> A(a, n, n, k), b(randomVec<T>(n * k, 52), n, 1, k), b0 = b;
    CholeskyBatchFactoriser<T> chol(A);
    chol.factorise();
    chol.solve(b);
    std::vector<T> x, bb;
    b.download(x);
    b0.download(bb);
    for (size_t i = 0; i < k; i++) {
        double num = 0, den = 0;
        for (size_t r = 0; r < n; r++) {
            double acc = 0;
            for (size_t c = 0; c < n; c++) acc += (double)a[i * n * n + c * n + r] * x[i * n + c];
            num += (acc - bb[i * n + r]) * (acc - bb[i * n + r]);
            den += (double)bb[i * n + r] * bb[i * n + r];
        }
        EXPECT_LT(std::sqrt(num / den), eps);
    }
}
TEST(choleskyBatchBeyond128) { choleskyBig<float>(200, 1e-4f); choleskyBig<double>(300, 1e-11); }

// CholeskyFactoriser on one large matrix (float: the blocked whole-GPU path
// with tensor-core trailing updates; double: one thread block): factorise,
// solve, residual of the solution against the original A.
template <typename T>
void choleskyLarge(size_t n, T eps) {
    std::vector<T> g = randomVec<T>(n * n, 61), a(n * n, T(0));
    for (size_t c = 0; c < n; c++)
        for (size_t r = 0; r < n; r++) {
            double acc = r == c ? 0.5 : 0.0;
            for (size_t l = 0; l < n; l++) acc += (double)g[r * n + l] * g[c * n + l] / n;
            a[c * n + r] = (T)acc;
        }
    DTensor<T> A(a, n, n, 1), b(randomVec<T>(n, 62), n, 1, 1), b0 = b;
    CholeskyFactoriser<T> chol(A);
    chol.factorise();
    EXPECT_EQ(chol.info()(0), 0);
    chol.solve(b);
    std::vector<T> x, bb, l;
    b.download(x);
    b0.download(bb);
    A.download(l);
    double num = 0, den = 0;
    for (size_t r = 0; r < n; r++) {
        double acc = 0;
        for (size_t c = 0; c < n; c++) acc += (double)a[c * n + r] * x[c];
        num += (acc - bb[r]) * (acc - bb[r]);
        den += (double)bb[r] * bb[r];
    }
    EXPECT_LT(std::sqrt(num / den), eps);
    bool upper_kept = true;  // the strict upper triangle is not written
    for (size_t c = 1; c < n; c++)
        for (size_t r = 0; r < c; r++) upper_kept = upper_kept && l[c * n + r] == a[c * n + r];
    EXPECT_TRUE(upper_kept);
}
TEST(choleskyFactoriserLarge) { choleskyLarge<float>(700, 1e-4f); choleskyLarge<double>(300, 1e-11); }

// GivensAnnihilatorBatched zeroes (k, j) of every matrix with its own rotation;
// applyLeftGivensRotationBatched with those coefficients reproduces it
template <typename T> static void givensBatched(T eps) {
    const size_t m = 5, n = 7, k = 9;
    std::vector<T> a = randomVec<T>(m * n * k, 61);
    DTensor<T> A(a, m, n, k), B(a, m, n, k);
    GivensAnnihilatorBatched<T> ga(A);
    ga.annihilate(1, 3, 2);
    std::vector<T> got;
    A.download(got);
    for (size_t i = 0; i < k; i++) EXPECT_LT(std::abs((double)got[i * m * n + 2 * m + 3]), eps);
    std::vector<T> co;
    ga.coefficients().download(co);
    std::vector<T> cv(k), sv(k);
    for (size_t i = 0; i < k; i++) { cv[i] = co[3 * i + 1]; sv[i] = co[3 * i + 2]; }
    DTensor<T> c(cv, 1, 1, k), s(sv, 1, 1, k);
    B.applyLeftGivensRotationBatched(1, 3, c, s);
    std::vector<T> got2;
    B.download(got2);
    double worst = 0;
    for (size_t e = 0; e < got.size(); e++) worst = std::max(worst, std::abs((double)got[e] - got2[e]));
    EXPECT_LT(worst, eps);
    EXPECT_THROW(ga.annihilate(2, 2, 0), std::invalid_argument);
    // right rotation of columns 0 and 4 of every matrix; column norms are preserved
    DTensor<T> C(a, m, n, k);
    C.applyRightGivensRotationBatched(0, 4, c, s);
    std::vector<T> got3;
    C.download(got3);
    for (size_t i = 0; i < k; i++) {
        double before = 0, after = 0;
        for (size_t r = 0; r < m; r++) {
            before += (double)a[i * m * n + r] * a[i * m * n + r] + (double)a[i * m * n + 4 * m + r] * a[i * m * n + 4 * m + r];
            after += (double)got3[i * m * n + r] * got3[i * m * n + r] +
                     (double)got3[i * m * n + 4 * m + r] * got3[i * m * n + 4 * m + r];
        }
        EXPECT_NEAR(before, after, eps * 100);
    }
}
TEST(givensBatchedExtension) { givensBatched<float>(PRECISION_LOW); givensBatched<double>(PRECISION_HIGH); }

int main(int argc, char **argv) {
    int failed_tests = 0;
    for (auto &t : registry()) {
        if (argc > 1 && t.name.find(argv[1]) == std::string::npos) continue;
        g_current = t.name;
        g_test_failed = false;
        try {
            t.fn();
        } catch (const std::exception &e) {
            g_test_failed = true;
            std::printf("  exception in %s: %s\n", t.name.c_str(), e.what());
        }
        std::printf("%s %s\n", g_test_failed ? "FAIL" : "PASS", t.name.c_str());
        failed_tests += g_test_failed;
    }
    std::printf("%d tests, %d failed, %d failed checks\n", (int)registry().size(), failed_tests, g_fail_checks);
    return failed_tests ? 1 : 0;
}
