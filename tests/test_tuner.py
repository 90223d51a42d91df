"""The serving engine's autotuner (csrc/tuner.hpp, host-only code) compiled
on its own with the host C++ compiler: warps per k-mode chosen from the
measured prior, by launch size when the GPU is otherwise idle and by the
whole load when it is shared, overridden by measurements, with every eighth
launch of a bucket exploring the runner-up."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "bolt.jl_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include "tuner.hpp"
int main() {
  const int nsm = 152;
  {  // isolated launches: size decides through the prior
    bolt::Tuner t;
    std::printf("iso_small %d\n", t.pick(false, 300, nsm));    // <= 2 modes/SM: lowest latency
    std::printf("iso_1200 %d\n", t.pick(false, 1200, nsm));    // 7.9 modes/SM: 4 warps cheapest
    std::printf("iso_4800 %d\n", t.pick(false, 4800, nsm));    // 31.6 modes/SM: 1 warp cheapest
  }
  {  // shared launches: the saturated prior, no one-wave shortcut
    bolt::Tuner t;
    std::printf("shared_small %d\n", t.pick(true, 300, nsm));
    std::printf("shared_1200 %d\n", t.pick(true, 1200, nsm));
  }
  {  // measurements of two variants that contradict the prior win
    bolt::Tuner t;
    t.update(false, 4800, 1, 10.0, 1e6);  // 1 warp: 1e-5 s per mode-step
    t.update(false, 4800, 4, 1.0, 1e6);   // 4 warps: 1e-6 s per mode-step
    std::printf("measured_4800 %d\n", t.pick(false, 4800, nsm));
    // the same bucket for a shared launch has its own table: still the prior
    std::printf("measured_shared_4800 %d\n", t.pick(true, 4800, nsm));
  }
  {  // every eighth pick of a bucket tries the runner-up
    bolt::Tuner t;
    int other = 0;
    for (int i = 1; i <= 16; ++i) other += t.pick(true, 4800, nsm) != 1;
    std::printf("explore %d\n", other);
  }
  {  // invalid measurements are ignored
    bolt::Tuner t;
    t.update(false, 4800, 4, 0.0, 1e6);
    t.update(false, 4800, 4, 1.0, 0.0);
    std::printf("ignored %d\n", t.pick(false, 4800, nsm));
  }
  return 0;
}
"""


def test_tuner_decisions(tmp_path):
    src = tmp_path / "tuner_harness.cpp"
    exe = tmp_path / "tuner_harness"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in
               subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines())
    assert out["iso_small"] == "4"
    assert out["iso_1200"] == "4"
    assert out["iso_4800"] == "1"
    assert out["shared_small"] == "1"
    assert out["shared_1200"] == "1"
    assert out["measured_4800"] == "4"
    assert out["measured_shared_4800"] == "1"
    assert out["explore"] == "2"
    assert out["ignored"] == "1"
