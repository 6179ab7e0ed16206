/* The reference's tensor-level C++ surface on libkvgpu: Block<Rank> and
 * Tensor<Rank> with norm / overlap / transpose / stack (holstein/block.h,
 * holstein/tensor.h), product<N1,N2,nc>, apply_zero / apply_single /
 * apply_double and env_sweep (holstein/product.h), local_krylov<Rank> with
 * KrylovConfig / KrylovExit (holstein/exponential.h) and svd_impl<R1,R2> with
 * SVDConfig (holstein/svd.h).  Header-only over the C ABI (include/kvgpu.h);
 * link with -lkvgpu.  The drop-in headers block.h, tensor.h, product.h,
 * exponential.h and svd.h of this directory include it, so code written
 * against those reference headers compiles unchanged.
 *
 * Where the data lives.  A Tensor's working copy is a device tensor: every
 * contraction, H_eff apply, environment update, Krylov exponential and SVD
 * takes its operands' device copies and returns a tensor that exists only on
 * the device, so a chain of such calls moves no block data between host and
 * device.  The blocks are copied to the host when the caller looks at them
 * (at, operator[], num_blocks, dirs, legs, norm, overlap, transpose,
 * arithmetic); a non-const access drops the device copy, and the next
 * device call uploads the host blocks again.  Copies of a Tensor share one
 * device copy, which no call modifies in place.
 *
 * Kept from the reference: names, template parameters and argument meaning;
 * blocks row-major in the reference's element order; Block::inner and
 * overlap(a, b) conjugate the second operand's blocks (zdotc, holstein/
 * tensor.h:224-237); the truncation rule and the folding of the singular
 * values of svd_impl; errors print a message and exit(1).
 * Differences: product takes opA in {NoTrans, ConjTrans} and opB in {NoTrans,
 * Trans} (the combinations the reference's sweeps use); env_sweep has the
 * MPO form and the two-leg bra/ket form; local_krylov's KrylovExit carries
 * the Krylov dimension, the exit reason derived from it (AchMaxItr when it
 * reached MaxIter - 1) and LossNorm, with KrylovErr NaN (the library does
 * not report the Lanczos error estimate); svd_impl takes LeftDir = -1 (the
 * value every reference sweep passes) and its SaveFile record lists the kept
 * singular values recovered as the norms of the folded factor's states.
 * KV_PRECISION=mixed selects the mixed-precision path, KV_DEVICE the GPU. */
#ifndef KV_HOLSTEIN_OPS_H
#define KV_HOLSTEIN_OPS_H

#include <algorithm>
#include <cmath>
#include <initializer_list>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <tuple>

#include "kv_holstein.h"

// CBLAS transpose flags (the values the reference passes to zgemm), unless a
// CBLAS or MKL header already declared them
#if !defined(KV_NO_CBLAS_ENUMS) && !defined(CBLAS_H) && !defined(__MKL_CBLAS_H__) && !defined(_MKL_TYPES_H_)
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
#endif

namespace KylinVib {
typedef std::initializer_list<INT> Brace;

namespace Holstein {
namespace detail {

inline void fail(const string &what) {
    cout << what << endl;
    exit(1);
}

template <size_t R>
size_t count(const array<INT, R> &sp) {
    size_t n = 1;
    for (INT s : sp) n *= (size_t)s;
    return n;
}

template <size_t R>
array<INT, R> from_brace(Brace b) {
    if (b.size() != R) fail("Brace of the wrong length");
    array<INT, R> a{};
    std::copy(b.begin(), b.end(), a.begin());
    return a;
}

}  // namespace detail

// ------------------------------------------------------------------ Block
// A dense complex128 block, row-major (holstein/block.h:23-166).
template <INT Rank>
class Block {
  public:
    Block() = default;
    Block(const array<INT, Rank> &Sp, const array<INT, Rank> &Qn)
        : shape_(Sp), qn_(Qn), data_(detail::count(Sp)) {
        make_distance();
    }
    Block(Brace Sp, Brace Qn) : Block(detail::from_brace<Rank>(Sp), detail::from_brace<Rank>(Qn)) {}

    INT size() const { return (INT)data_.size(); }
    Complex *ptr() { return data_.data(); }
    const Complex *cptr() const { return data_.data(); }
    const array<INT, Rank> &shape() const { return shape_; }
    const array<INT, Rank> &dist() const { return dist_; }
    const array<INT, Rank> &qn() const { return qn_; }

    Block &operator+=(const Block &rhs) {
        if (rhs.data_.size() != data_.size()) detail::fail("Block += of different sizes");
        for (size_t i = 0; i < data_.size(); ++i) data_[i] += rhs.data_[i];
        return *this;
    }
    Block operator*(const Complex &val) const {
        Block res(*this);
        for (auto &x : res.data_) x *= val;
        return res;
    }
    Block &operator*=(double val) {
        for (auto &x : data_) x *= val;
        return *this;
    }
    Complex &operator()(const array<INT, Rank> &idx) {
        const INT pos = std::inner_product(idx.begin(), idx.end(), dist_.begin(), (INT)0);
        if (pos < 0 || pos >= size()) detail::fail("Overflow!");
        return data_[(size_t)pos];
    }
    Complex &operator()(Brace idx) { return (*this)(detail::from_brace<Rank>(idx)); }

    // Frobenius norm, and sum conj(this) . oth (zdotc)
    double norm() const {
        double s = 0.0;
        for (const auto &x : data_) s += std::norm(x);
        return std::sqrt(s);
    }
    Complex inner(const Block &oth) const {
        Complex s = 0.0;
        const size_t n = std::min(data_.size(), oth.data_.size());
        for (size_t i = 0; i < n; ++i) s += std::conj(data_[i]) * oth.data_[i];
        return s;
    }

    void make_distance() {
        dist_[Rank - 1] = 1;
        for (INT i = Rank - 2; i >= 0; --i) dist_[i] = dist_[i + 1] * shape_[i + 1];
    }

  private:
    array<INT, Rank> shape_{}, dist_{}, qn_{};
    vector<Complex> data_;
};

// ----------------------------------------------------------------- Tensor
// A U(1) block-sparse tensor (holstein/tensor.h:16-209); see the file header
// for where its blocks live.
template <INT Rank>
class Tensor {
  public:
    Tensor() = default;
    Tensor(const array<map<INT, INT>, Rank> &Legs, const array<INT, Rank> &Di) : leg_(Legs), dirs_(Di) {}
    Tensor(const array<map<INT, INT>, Rank> &Legs, const array<INT, Rank> &Di, INT NumBks)
        : leg_(Legs), dirs_(Di), blocks_((size_t)NumBks) {}
    explicit Tensor(const array<INT, Rank> &Di) : dirs_(Di) {}
    Tensor(Brace Di) : dirs_(detail::from_brace<Rank>(Di)) {}

    // a tensor held by the library (takes ownership of the handle)
    static Tensor adopt(kv_tensor t) {
        Tensor r;
        r.dev_ = std::shared_ptr<kv_tensor_s>(t, [](kv_tensor p) { kv_tensor_free(p); });
        r.host_ = false;
        return r;
    }
    // the device copy (uploaded from the host blocks if there is none); owned by *this
    kv_tensor device() const {
        if (!dev_) {
            detail::ensure_init();
            vector<int> sh, q;
            vector<double> d;
            for (const auto &b : blocks_) {
                sh.insert(sh.end(), b.shape().begin(), b.shape().end());
                q.insert(q.end(), b.qn().begin(), b.qn().end());
                const double *p = reinterpret_cast<const double *>(b.cptr());
                d.insert(d.end(), p, p + 2 * (size_t)b.size());
            }
            kv_tensor t = nullptr;
            detail::check(kv_tensor_create(Rank, dirs_.data(), (int)blocks_.size(), sh.data(), q.data(), d.data(), &t),
                          "kv_tensor_create");
            dev_ = std::shared_ptr<kv_tensor_s>(t, [](kv_tensor p) { kv_tensor_free(p); });
        }
        return dev_.get();
    }

    // --------------------------------------------- reference accessors
    const map<INT, INT> &cleg(INT axis) const {
        fetch();
        return leg_[axis];
    }
    const array<map<INT, INT>, Rank> &clegs() const {
        fetch();
        return leg_;
    }
    map<INT, INT> &leg(INT axis) {
        fetch();
        return leg_[axis];
    }
    INT num_blocks() const {
        fetch();
        return (INT)blocks_.size();
    }
    const array<INT, Rank> &dirs() const {
        fetch();
        return dirs_;
    }
    Block<Rank> &operator[](INT i) {
        touch();
        return blocks_[(size_t)i];
    }
    const Block<Rank> &at(INT i) const {
        fetch();
        return blocks_[(size_t)i];
    }
    void push_back(const Block<Rank> &t) {
        touch();
        blocks_.push_back(t);
    }
    // add into a block of the same shape and charges, else append
    void push_back_ch(const Block<Rank> &t) {
        touch();
        for (auto &b : blocks_)
            if (b.shape() == t.shape() && b.qn() == t.qn()) {
                b += t;
                return;
            }
        blocks_.push_back(t);
    }
    void check_legs() {
        fetch();
        for (const auto &b : blocks_)
            for (INT j = 0; j < Rank; ++j) leg_[j][b.qn()[j]] = b.shape()[j];
    }
    void check_sym(const char *var) const {
        fetch();
        for (size_t i = 0; i < blocks_.size(); ++i) {
            const INT s = std::inner_product(dirs_.begin(), dirs_.end(), blocks_[i].qn().begin(), 0);
            if (s != 0) {
                cout << "Tensor " << var << " has symmetry-destroyed blocks at index " << i << endl;
                break;
            }
        }
    }

    Tensor &operator+=(const Tensor &rhs) {
        for (INT i = 0; i < rhs.num_blocks(); ++i) push_back_ch(rhs.at(i));
        return *this;
    }
    Tensor operator*(const Complex &val) const {
        fetch();
        Tensor res(leg_, dirs_);
        for (const auto &b : blocks_) res.blocks_.push_back(b * val);
        return res;
    }
    Tensor &operator*=(double val) {
        touch();
        for (auto &b : blocks_) b *= val;
        return *this;
    }

  private:
    // bring the blocks (and dirs, legs) to the host from the device copy
    void fetch() const {
        if (host_) return;
        int rank = 0, nb = 0;
        long long ne = 0;
        detail::check(kv_tensor_info(dev_.get(), &rank, &nb, &ne), "kv_tensor_info");
        if (rank != Rank) detail::fail("unexpected tensor rank " + to_string(rank));
        vector<int> sh((size_t)nb * Rank), q((size_t)nb * Rank);
        vector<double> d(2 * (size_t)ne + 2);
        detail::check(kv_tensor_download(dev_.get(), dirs_.data(), sh.data(), q.data(), d.data()),
                      "kv_tensor_download");
        blocks_.clear();
        size_t off = 0;
        for (int j = 0; j < nb; ++j) {
            array<INT, Rank> s{}, c{};
            for (INT i = 0; i < Rank; ++i) {
                s[i] = sh[(size_t)j * Rank + i];
                c[i] = q[(size_t)j * Rank + i];
            }
            Block<Rank> b(s, c);
            const size_t n = (size_t)b.size();
            for (size_t k = 0; k < n; ++k) b.ptr()[k] = Complex(d[2 * (off + k)], d[2 * (off + k) + 1]);
            off += n;
            for (INT i = 0; i < Rank; ++i) leg_[i][c[i]] = s[i];
            blocks_.push_back(std::move(b));
        }
        host_ = true;
    }
    // the host blocks are about to change: the device copy is no longer current
    void touch() {
        fetch();
        dev_.reset();
    }

    mutable array<map<INT, INT>, Rank> leg_;
    mutable array<INT, Rank> dirs_{};
    mutable vector<Block<Rank>> blocks_;
    mutable bool host_ = true;                  // blocks_ holds the current blocks
    mutable std::shared_ptr<kv_tensor_s> dev_;  // the current device copy, if any
};

// host copy of a tensor read by the drop-in State / Operator loaders
template <INT Rank>
Tensor<Rank> to_tensor(const HostTensor<Rank> &h) {
    Tensor<Rank> t(h.dirs);
    for (INT j = 0; j < h.num_blocks(); ++j) {
        Block<Rank> b(h.shape[j], h.qn[j]);
        std::copy(h.data[j].begin(), h.data[j].end(), b.ptr());
        t.push_back(b);
    }
    t.check_legs();
    return t;
}

// the host blocks of a tensor in the drop-in State / Operator form
template <INT Rank>
HostTensor<Rank> to_host(const Tensor<Rank> &t) {
    HostTensor<Rank> h;
    h.dirs = t.dirs();
    for (INT j = 0; j < t.num_blocks(); ++j) {
        const Block<Rank> &b = t.at(j);
        h.shape.push_back(b.shape());
        h.qn.push_back(b.qn());
        h.data.emplace_back(b.cptr(), b.cptr() + b.size());
    }
    return h;
}

// om2 added into om1 as a direct sum along the legs ax (holstein/tensor.h
// stack, :263-320); om2 is left unchanged
template <INT Rank>
void stack(Tensor<Rank> &om1, const Tensor<Rank> &om2, Brace ax) {
    HostTensor<Rank> h = to_host(om1);
    detail::stack_into(h, to_host(om2), vector<int>(ax.begin(), ax.end()));
    om1 = to_tensor(h);
}

// sqrt of the summed squared block norms (holstein/tensor.h:214-223)
template <INT Rank>
double norm(const Tensor<Rank> &ori) {
    double s = 0.0;
    for (INT i = 0; i < ori.num_blocks(); ++i) s += std::pow(ori.at(i).norm(), 2.0);
    return std::sqrt(s);
}

// sum over blocks of equal shape and charges of conj(oth) . ori
// (holstein/tensor.h:225-241)
template <INT Rank>
Complex overlap(const Tensor<Rank> &ori, const Tensor<Rank> &oth) {
    Complex s = 0.0;
    for (INT i = 0; i < ori.num_blocks(); ++i)
        for (INT j = 0; j < oth.num_blocks(); ++j)
            if (ori.at(i).shape() == oth.at(j).shape() && ori.at(i).qn() == oth.at(j).qn())
                s += oth.at(j).inner(ori.at(i));
    return s;
}

// legs permuted: result leg i is leg ax[i] (holstein/tensor.h:244-260)
template <INT Rank>
Tensor<Rank> transpose(const Tensor<Rank> &ori, Brace ax) {
    const array<INT, Rank> p = detail::from_brace<Rank>(ax);
    array<map<INT, INT>, Rank> legs;
    array<INT, Rank> di{};
    for (INT i = 0; i < Rank; ++i) {
        legs[i] = ori.cleg(p[i]);
        di[i] = ori.dirs()[p[i]];
    }
    Tensor<Rank> res(legs, di);
    for (INT b = 0; b < ori.num_blocks(); ++b) {
        const Block<Rank> &o = ori.at(b);
        array<INT, Rank> sp{}, qn{};
        for (INT i = 0; i < Rank; ++i) {
            sp[i] = o.shape()[p[i]];
            qn[i] = o.qn()[p[i]];
        }
        Block<Rank> r(sp, qn);
        for (INT e = 0; e < o.size(); ++e) {
            array<INT, Rank> idx{};
            for (INT j = 0; j < Rank; ++j) idx[j] = e / o.dist()[p[j]] % o.shape()[p[j]];
            r(idx) = o.cptr()[e];
        }
        res.push_back(r);
    }
    return res;
}

// ---------------------------------------------------------- contractions
// product<N1,N2,nc>: the last nc legs of op(m1) with the first nc of op(m2)
// (holstein/product.h:61-201)
template <INT N1, INT N2, INT nc>
Tensor<N1 + N2 - 2 * nc> product(const Tensor<N1> &m1, const Tensor<N2> &m2, CBLAS_TRANSPOSE T1, CBLAS_TRANSPOSE T2) {
    static_assert(nc >= 1 && nc <= N1 && nc <= N2 && N1 + N2 - 2 * nc >= 1, "contraction ranks");
    kv_tensor a = m1.device(), b = m2.device(), out = nullptr;
    detail::check(kv_product(a, b, nc, (int)T1, (int)T2, detail::precision(), &out), "product");
    return Tensor<N1 + N2 - 2 * nc>::adopt(out);
}

// H_eff . C for a zero-site centre (holstein/product.h:540-545)
inline Tensor<2> apply_zero(const Tensor<3> &envL, const Tensor<2> &C, const Tensor<3> &envR) {
    kv_tensor out = nullptr;
    detail::check(kv_heff_apply(0, envL.device(), C.device(), nullptr, nullptr, envR.device(), 1.0,
                                detail::precision(), &out),
                  "apply_zero");
    return Tensor<2>::adopt(out);
}

// H_eff . A for one site (holstein/product.h:547-553)
inline Tensor<3> apply_single(const Tensor<3> &envL, const Tensor<3> &mps, const Tensor<4> &mpo,
                              const Tensor<3> &envR) {
    kv_tensor out = nullptr;
    detail::check(kv_heff_apply(1, envL.device(), mps.device(), mpo.device(), nullptr, envR.device(), 1.0,
                                detail::precision(), &out),
                  "apply_single");
    return Tensor<3>::adopt(out);
}

// H_eff . AA for two sites (holstein/product.h:478-486)
inline Tensor<4> apply_double(const Tensor<3> &envL, const Tensor<4> &mps, const Tensor<4> &mpo1,
                              const Tensor<4> &mpo2, const Tensor<3> &envR) {
    kv_tensor out = nullptr;
    detail::check(kv_heff_apply(2, envL.device(), mps.device(), mpo1.device(), mpo2.device(), envR.device(), 1.0,
                                detail::precision(), &out),
                  "apply_double");
    return Tensor<4>::adopt(out);
}

// environment one site further (holstein/product.h:488-503)
inline Tensor<3> env_sweep(const Tensor<3> &env, const Tensor<3> &mps, const Tensor<4> &mpo, bool Left2Right) {
    kv_tensor out = nullptr;
    detail::check(kv_env_update(Left2Right ? 1 : 0, env.device(), mps.device(), mpo.device(), detail::precision(),
                                &out),
                  "env_sweep");
    return Tensor<3>::adopt(out);
}

// bra/ket overlap environment one site further (holstein/product.h:523-538)
inline Tensor<2> env_sweep(const Tensor<2> &env, const Tensor<3> &mps1, const Tensor<3> &mps2,
                           bool Left2Right = true) {
    if (!Left2Right)
        return env_sweep(env, transpose<3>(mps1, {2, 1, 0}), transpose<3>(mps2, {2, 1, 0}), true);
    Tensor<3> lm = product<2, 3, 1>(env, mps2, CblasNoTrans, CblasNoTrans);
    return product<3, 3, 2>(mps1, lm, CblasConjTrans, CblasNoTrans);
}

// ---------------------------------------------------------------- Krylov
enum class KrylovExitReason { AchKryThr, AchMaxItr };

struct KrylovConfig {
    double KrylovThres = 1.0e-9;
    INT MaxIter = 15;
    double TimeStep = 0.0;
};

struct KrylovExit {
    KrylovExitReason reason = KrylovExitReason::AchKryThr;
    double KrylovErr = std::numeric_limits<double>::quiet_NaN();  // not reported by the library
    INT RealIter = 0;
    double LossNorm = 0.0;
};

// mps <- exp(-+i H_eff TimeStep/2) mps / |mps| by Lanczos on the device
// (holstein/exponential.h:92-190); Rank 2, 3, 4 = zero-, one-, two-site
// (the MPOs a rank does not use are not read)
template <INT Rank>
KrylovExit local_krylov(const Tensor<3> &envl, Tensor<Rank> &mps, const Tensor<4> &mpo1, const Tensor<4> &mpo2,
                        const Tensor<3> &envr, KrylovConfig &r, bool ReverseEvl = false) {
    static_assert(Rank >= 2 && Rank <= 4, "local_krylov acts on a zero-, one- or two-site centre");
    constexpr int nsite = Rank - 2;
    kv_tensor out = nullptr;
    int iters = 0;
    detail::check(kv_lanczos_expm(nsite, envl.device(), mps.device(), nsite >= 1 ? mpo1.device() : nullptr,
                                  nsite == 2 ? mpo2.device() : nullptr, envr.device(), r.TimeStep, r.MaxIter,
                                  r.KrylovThres, ReverseEvl ? 1 : 0, detail::precision(), &out, &iters),
                  "local_krylov");
    mps = Tensor<Rank>::adopt(out);
    KrylovExit ex;
    ex.RealIter = iters;
    ex.reason = iters >= r.MaxIter - 1 ? KrylovExitReason::AchMaxItr : KrylovExitReason::AchKryThr;
    ex.LossNorm = 1.0 - norm(mps);
    return ex;
}

// ------------------------------------------------------------------- SVD
struct SVDConfig {
    double SVDThres = 1.0e-9;
    INT MaxDim = 2000;
    double SAModeBeta = 0.1;
    bool Left2Right = true;
    bool EnableRenorm = false;
    bool EnableRescale = false;
};

namespace detail {

// singular values folded into a factor: the norms of its states (the last
// leg of U, the first leg of V), largest first
template <INT Rank>
vector<double> state_norms(const Tensor<Rank> &t, bool last_leg) {
    map<pair<INT, INT>, double> acc;  // (charge, index within the charge) -> sum |x|^2
    for (INT b = 0; b < t.num_blocks(); ++b) {
        const Block<Rank> &blk = t.at(b);
        const INT leg = last_leg ? Rank - 1 : 0;
        for (INT e = 0; e < blk.size(); ++e) {
            const INT k = e / blk.dist()[leg] % blk.shape()[leg];
            acc[{blk.qn()[leg], k}] += std::norm(blk.cptr()[e]);
        }
    }
    vector<double> s;
    for (auto &kv : acc) s.push_back(std::sqrt(kv.second));
    std::sort(s.begin(), s.end(), [](double x, double y) { return x > y; });
    return s;
}

}  // namespace detail

// block SVD per charge sector with the global truncation, singular values
// folded into the right factor (Left2Right) or the left one
// (holstein/svd.h:296-440)
template <INT R1, INT R2>
std::tuple<Tensor<R1 + 1>, Tensor<R2 + 1>> svd_impl(Tensor<R1 + R2> &A, SVDConfig &r, INT LeftDir,
                                                     bool PrintTrunc = false, bool SaveFile = false) {
    if (LeftDir != -1) detail::fail("svd_impl: only LeftDir = -1 is supported");
    kv_tensor U = nullptr, V = nullptr;
    int kept = 0, total = 0;
    detail::check(kv_svd_truncate(A.device(), R1, r.Left2Right ? 1 : 0, r.SVDThres, r.MaxDim, detail::precision(), &U,
                                  &V, &kept, &total),
                  "svd_impl");
    Tensor<R1 + 1> Lef = Tensor<R1 + 1>::adopt(U);
    Tensor<R2 + 1> Rig = Tensor<R2 + 1>::adopt(V);
    if (SaveFile) {
        const vector<double> s =
            r.Left2Right ? detail::state_norms(Rig, false) : detail::state_norms(Lef, true);
        ofstream ofs("SVS", ofstream::app);
        ofs << s.size() << endl;
        for (size_t i = 2; i < s.size(); ++i)
            ofs << std::left << setw(20) << std::scientific << setprecision(11)
                << log10(s[i] * s[i - 2] / pow(s[i - 1], 2.0)) << endl;
    }
    if (PrintTrunc) cout << total << " -> " << kept << endl;
    if (r.EnableRenorm) {
        if (r.Left2Right) Rig *= 1.0 / norm(Rig);
        else Lef *= 1.0 / norm(Lef);
    }
    if (r.EnableRescale) {
        if (r.Left2Right) {
            const double n = norm(Rig);
            Rig *= pow(n, -0.5);
            Lef *= pow(n, 0.5);
        } else {
            const double n = norm(Lef);
            Lef *= pow(n, -0.5);
            Rig *= pow(n, 0.5);
        }
    }
    return std::make_tuple(Lef, Rig);
}

}  // namespace Holstein
}  // namespace KylinVib

#endif
