// Runs the drop-in headers' index maps and planner helpers on cases read
// from standard input, one per line, and prints one result line per case.
// tests/test_dropin_headers.py compares the lines with the reference's own
// functions (oracle/_ref). Host only: no device is touched.
//
//   sdl|shd n l[n] L[n] lb[n]          strided_(hierarchical_)domain_from_level
//   rsd n f[n] e[n] s[n] bf[n] be[n]    restrict_strided_with_discrete
//   rtd fwd l lmin L lf le wavelet      get_required_transform_domain (1D)
//   pui n                               initialize_dim_periodic_unit_interval
//   ihs n l[n]                          iterate_hierarchical_subspaces
//   cpb period k i[k]                   covering_periodic_bounds
//   pps wmin wmax origin l L pl         pole_pass_segments
//   rpb f0 f1 e0 e1 s0 s1 bmin bmax P   restrict_periodic_bounds<dim 0> (2D)
//   ftb L k (min max)[k]                for_each_transform_index
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <paliwa/paliwa_dimensions.hpp>
#include <paliwa/paliwa_domains.hpp>
#include <paliwa/paliwa_utils.hpp>

using namespace paliwa;

template <class... D> struct Tags {};

template <class F> void with_rank(int n, F &&f) {
  switch (n) {
  case 1: return f(Tags<DDimA>{});
  case 2: return f(Tags<DDimA, DDimB>{});
  case 3: return f(Tags<DDimA, DDimB, DDimC>{});
  case 4: return f(Tags<DDimA, DDimB, DDimC, DDimD>{});
  }
  throw std::invalid_argument("rank");
}

template <std::size_t N> std::array<long, N> read_arr(std::istream &in) {
  std::array<long, N> a{};
  for (auto &x : a) in >> x;
  return a;
}

template <class... D>
void print_domain(ddc::StridedDiscreteDomain<D...> const &d) {
  ((std::cout << d.front().template uid<D>() << ' '), ...);
  ((std::cout << d.extents().template get<D>() << ' '), ...);
  ((std::cout << d.strides().template get<D>() << ' '), ...);
}

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    std::string cmd;
    in >> cmd;
    try {
      if (cmd == "sdl" || cmd == "shd") {
        int n;
        in >> n;
        with_rank(n, [&]<class... D>(Tags<D...>) {
          constexpr std::size_t N = sizeof...(D);
          auto const l = read_arr<N>(in), L = read_arr<N>(in),
                     lb = read_arr<N>(in);
          ddc::DiscreteElement<D...> const b(lb);
          print_domain(cmd == "sdl"
                           ? strided_domain_from_level<D...>(l, L, b)
                           : strided_hierarchical_domain_from_level<D...>(
                                 l, L, b));
        });
      } else if (cmd == "rsd") {
        int n;
        in >> n;
        with_rank(n, [&]<class... D>(Tags<D...>) {
          constexpr std::size_t N = sizeof...(D);
          auto const f = read_arr<N>(in), e = read_arr<N>(in),
                     s = read_arr<N>(in), bf = read_arr<N>(in),
                     be = read_arr<N>(in);
          ddc::StridedDiscreteDomain<D...> const dom{
              ddc::DiscreteElement<D...>(f), ddc::DiscreteVector<D...>(e),
              ddc::DiscreteVector<D...>(s)};
          ddc::DiscreteDomain<D...> const box{ddc::DiscreteElement<D...>(bf),
                                              ddc::DiscreteVector<D...>(be)};
          print_domain(restrict_strided_with_discrete(dom, box));
        });
      } else if (cmd == "rtd") {
        long fwd, l, lmin, L, lf, le;
        std::string w;
        in >> fwd >> l >> lmin >> L >> lf >> le >> w;
        using Dm = DDimA;
        auto const full = strided_domain_from_level<Dm>(
            std::array<long, 1>{l}, std::array<long, 1>{L});
        ddc::DiscreteDomain<Dm> const local{ddc::DiscreteElement<Dm>(lf),
                                            ddc::DiscreteVector<Dm>(le)};
        auto const g = get_required_transform_domain<Dm>(
            fwd != 0, full, local, ddc::DiscreteVector<Dm>(l),
            ddc::DiscreteVector<Dm>(lmin), ddc::DiscreteVector<Dm>(L), w);
        for (auto it = g.begin(); it != g.end(); ++it)
          std::cout << (*it).uid() << ' ';
      } else if (cmd == "pui") {
        long n;
        in >> n;
        struct Probe {};
        using Dm = D_Dim<Probe, 9>;
        auto const dom = initialize_dim_periodic_unit_interval<Dm>(
            ddc::DiscreteVector<Dm>(n));
        std::cout.precision(17);
        ddc::host_for_each(dom, [&](ddc::DiscreteElement<Dm> e) {
          std::cout << double(ddc::coordinate(e)) << ' ';
        });
      } else if (cmd == "ihs") {
        int n;
        in >> n;
        std::vector<long> nodal(n), tmp(n, 0);
        for (auto &x : nodal) in >> x;
        iterate_hierarchical_subspaces<std::vector<long>>(
            nodal, tmp, 0, [](std::vector<long> const &s) {
              for (long x : s) std::cout << x << ',';
              std::cout << ' ';
            });
      } else if (cmd == "cpb") {
        long period, k;
        in >> period >> k;
        std::vector<long> idx(k);
        for (auto &x : idx) in >> x;
        auto const b = covering_periodic_bounds(idx, period);
        std::cout << b.min << ' ' << b.max;
      } else if (cmd == "pps") {
        long wmin, wmax, origin;
        int l, L, pl;
        in >> wmin >> wmax >> origin >> l >> L >> pl;
        for (auto const &s : pole_pass_segments(
                 {wmin, wmax}, static_cast<std::size_t>(origin), l, L, pl))
          std::cout << s.first << ',' << s.count << ',' << s.stride << ','
                    << s.lower << ',' << s.upper << ' ';
      } else if (cmd == "rpb") {
        long f0, f1, e0, e1, s0, s1, bmin, bmax, P;
        in >> f0 >> f1 >> e0 >> e1 >> s0 >> s1 >> bmin >> bmax >> P;
        using D2 = ddc::StridedDiscreteDomain<DDimA, DDimB>;
        D2 const dom{ddc::DiscreteElement<DDimA, DDimB>(f0, f1),
                     ddc::DiscreteVector<DDimA, DDimB>(e0, e1),
                     ddc::DiscreteVector<DDimA, DDimB>(s0, s1)};
        for (auto const &d :
             restrict_periodic_bounds<DDimA>(dom, {bmin, bmax}, P)) {
          print_domain(d);
          std::cout << "| ";
        }
      } else if (cmd == "ftb") {
        long L, k;
        in >> L >> k;
        std::vector<PeriodicBounds> b(k);
        for (auto &x : b) in >> x.min >> x.max;
        for_each_transform_index<DDimA>(b, L, [](ddc::DiscreteElement<DDimA> e) {
          std::cout << e.uid() << ' ';
        });
      } else {
        std::cout << "?";
      }
    } catch (std::exception const &e) {
      std::cout << "error " << typeid(e).name();
    }
    std::cout << '\n';
  }
  return 0;
}
