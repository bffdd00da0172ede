// C++ drop-in check: a libParanumal-style caller of include/ogs.hpp, written
// like dawgs' CorrectnessTest (dawgsMain.cpp:314-416): build box-mesh ids, set
// up an Unsigned handle and a Signed unique handle, run device and host
// GatherScatter and device Gather+Scatter, and compare each result entry by
// entry with a brute-force fold over the id groups in ascending local order.
#include <cmath>
#include <cstdio>
#include <map>
#include <vector>

#include "ogs.hpp"

using namespace libp;

static memory<hlong> make_ids(int NX, int NY, int NZ, int p) {
  const int Nq = p + 1, Np = Nq * Nq * Nq;
  memory<hlong> ids(static_cast<size_t>(NX) * NY * NZ * Np);
  for (int K = 0; K < NZ; ++K)
    for (int J = 0; J < NY; ++J)
      for (int I = 0; I < NX; ++I) {
        hlong* e = ids.ptr() + static_cast<size_t>(I + J * NX + K * NX * NY) * Np;
        const hlong base = hlong(I) * p + hlong(J) * p * (p * NX + 1) +
                           hlong(K) * p * (p * NX + 1) * (p * NY + 1) + 1;
        for (int k = 0; k < Nq; ++k)
          for (int j = 0; j < Nq; ++j)
            for (int i = 0; i < Nq; ++i)
              e[i + j * Nq + k * Nq * Nq] = i + hlong(j) * (p * NX + 1) + hlong(k) * (p * NX + 1) * (p * NY + 1) + base;
      }
  return ids;
}

int main() {
  platform_t platform;
  comm_t comm;
  const int p = 3;
  memory<hlong> ids = make_ids(6, 5, 4, p);
  const dlong N = static_cast<dlong>(ids.length());

  memory<double> q(N);
  for (dlong n = 0; n < N; ++n) q[n] = std::sin(0.37 * n) * 0.25;

  // expected: fold each |id| group in ascending local index, starting from 0
  std::map<hlong, double> sum;
  for (dlong n = 0; n < N; ++n) sum[ids[n]] = 0.0;
  for (dlong n = 0; n < N; ++n) sum[ids[n]] += q[n];
  memory<double> qcheck(N);
  for (dlong n = 0; n < N; ++n) qcheck[n] = sum[ids[n]];

  int fails = 0;
  auto check = [&](const char* what, const memory<double>& got) {
    double err = 0.0;
    for (dlong n = 0; n < N; ++n) err += std::fabs(got[n] - qcheck[n]);
    const bool exact = std::memcmp(got.ptr(), qcheck.ptr(), sizeof(double) * N) == 0;
    std::printf("%-26s Error = %g%s\n", what, err, exact ? " (bit-exact)" : "");
    if (!exact) fails++;
  };

  try {
    ogs::ogs_t gs;
    gs.Setup(N, ids, comm, ogs::Unsigned, ogs::Auto, false, true, platform);
    ogs::ogs_t sgs;
    memory<hlong> sids(N);
    sids.copyFrom(ids);
    sgs.Setup(N, sids, comm, ogs::Signed, ogs::Auto, true, false, platform);
    std::printf("N = %d, NgatherGlobal = %lld, Ngather(unique) = %d\n", N, gs.NgatherGlobal, sgs.Ngather);

    deviceMemory<double> o_q = platform.malloc<double>(N, q);
    gs.GatherScatter(o_q, 1, ogs::Add, ogs::Sym);
    memory<double> qtest(N);
    o_q.copyTo(qtest);
    check("Device GatherScatter:", qtest);

    qtest.copyFrom(q);
    gs.GatherScatter(qtest, 1, ogs::Add, ogs::Sym);
    check("Host   GatherScatter:", qtest);

    o_q.copyFrom(q);
    deviceMemory<double> o_gq = platform.malloc<double>(sgs.Ngather);
    sgs.Gather(o_gq, o_q, 1, ogs::Add, ogs::Trans);
    sgs.Scatter(o_q, o_gq, 1, ogs::NoTrans);
    o_q.copyTo(qtest);
    check("Device Gather+Scatter:", qtest);

    memory<double> gq(sgs.Ngather);
    sgs.Gather(gq, q, 1, ogs::Add, ogs::Trans);
    sgs.Scatter(qtest, gq, 1, ogs::NoTrans);
    check("Host   Gather+Scatter:", qtest);

    // a copy shares the handle (ogsBase.hpp:80-82 shared_ptr members)
    ogs::ogs_t copy = gs;
    gs.Free();
    o_q.copyFrom(q);
    copy.GatherScatter(o_q, 1, ogs::Add, ogs::Sym);
    o_q.copyTo(qtest);
    check("Copied handle GS:", qtest);

    // the rejection the reference raises with LIBP_ABORT (ogsSetup.cpp:98-100)
    bool threw = false;
    try {
      ogs::ogs_t bad;
      bad.Setup(N, ids, comm, ogs::Unsigned, ogs::Auto, true, false, platform);
    } catch (const libp::exception& e) {
      threw = true;
      std::printf("rejected Unsigned+unique: %s\n", e.what());
    }
    if (!threw) fails++;

    memory<dlong> g2l(N);
    sgs.SetupGlobalToLocalMapping(g2l);
    for (dlong n = 0; n < N; ++n)
      if (g2l[n] < 0 || g2l[n] >= sgs.NlocalT) { fails++; break; }

    // halo_t at one rank (ogsHalo.cpp): no halo rows, Exchange and Combine
    // leave the vector as it is; the ids need one positive member per group
    ogs::halo_t halo;
    halo.Setup(N, sids, comm, ogs::Auto, false, platform);
    o_q.copyFrom(q);
    halo.Exchange(o_q, 1);
    halo.CombineStart(o_q, 1);
    halo.CombineFinish(o_q, 1);
    o_q.copyTo(qtest);
    qtest.copyFrom(q);
    halo.Exchange(qtest, 1);
    for (dlong n = 0; n < N; ++n)
      if (qtest[n] != q[n]) { fails++; break; }
    if (halo.Nhalo != 0 || halo.NhaloT != 0) fails++;
    ogs::halo_t ghalo;
    ghalo.SetupFromGather(sgs);
    ghalo.Exchange(o_gq, 1);
    threw = false;
    try {
      ogs::halo_t bad;
      bad.Setup(N, ids, comm, ogs::Auto, false, platform);  // every member positive
    } catch (const libp::exception& e) {
      threw = true;
      std::printf("rejected halo ids: %s\n", e.what());
    }
    if (!threw) fails++;
  } catch (const std::exception& e) {
    std::printf("exception: %s\n", e.what());
    return 2;
  }
  std::printf(fails ? "FAILED\n" : "PASSED\n");
  return fails ? 1 : 0;
}
