// admission_test.cpp -- unit test of the stitch server's admission policy
// (hm-cupano_gb300/csrc/hmp_admission.h); host only, run by tests/test_server_admission.py.
#include <cstdio>

#include "hmp_admission.h"

using hmp::AdmissionPolicy;

static int failures = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);            \
      ++failures;                                                 \
    }                                                             \
  } while (0)

int main() {
  {  // first request of a configuration creates; an idle instance is reused
    AdmissionPolicy p(100, 2);
    AdmissionPolicy::Decision d = p.decide(0, 40);
    CHECK(d.kind == AdmissionPolicy::kCreate && d.evict.empty());
    const int a = p.add(0, 40);
    d = p.decide(0, 40);
    CHECK(d.kind == AdmissionPolicy::kUse && d.instance == a);
    p.acquire(a);
    d = p.decide(0, 40);  // busy: a second instance fits
    CHECK(d.kind == AdmissionPolicy::kCreate);
    const int b = p.add(0, 40);
    p.acquire(b);
    d = p.decide(0, 40);  // per-configuration limit reached
    CHECK(d.kind == AdmissionPolicy::kWait);
    CHECK(p.resident() == 80 && p.peak() == 80);
  }
  {  // eviction: least recently used idle instances of other configurations go first
    AdmissionPolicy p(100, 4);
    const int a = p.add(0, 30);
    const int b = p.add(1, 30);
    const int c = p.add(2, 30);
    p.acquire(b);
    p.release(b);  // b used after a and c were created: c is older than b, a oldest
    p.acquire(c);
    p.release(c);
    AdmissionPolicy::Decision d = p.decide(3, 50);  // needs 40 more than free (10)
    CHECK(d.kind == AdmissionPolicy::kCreate);
    CHECK(d.evict.size() == 2 && d.evict[0] == a && d.evict[1] == b);
    for (int e : d.evict) p.remove(e);
    p.add(3, 50);
    CHECK(p.resident() == 80);
  }
  {  // busy instances are never evicted: the request waits
    AdmissionPolicy p(100, 4);
    const int a = p.add(0, 60);
    p.acquire(a);
    AdmissionPolicy::Decision d = p.decide(1, 50);
    CHECK(d.kind == AdmissionPolicy::kWait && d.evict.empty());
    p.release(a);
    d = p.decide(1, 50);
    CHECK(d.kind == AdmissionPolicy::kCreate && d.evict.size() == 1 && d.evict[0] == a);
  }
  {  // a configuration larger than the whole budget never fits
    AdmissionPolicy p(100, 4);
    CHECK(p.decide(0, 150).kind == AdmissionPolicy::kWait);
  }
  {  // removed slots are reused and the accounting stays exact
    AdmissionPolicy p(100, 4);
    const int a = p.add(0, 10);
    p.add(1, 20);
    p.remove(a);
    const int c = p.add(2, 30);
    CHECK(c == a);
    CHECK(p.resident() == 50 && p.peak() == 50);
  }
  std::printf(failures ? "FAILED %d\n" : "OK\n", failures);
  return failures ? 1 : 0;
}
