// Simulation clock handed to the callbacks (reference: include/prismspf/core/simulation_timer.h:12-82).
// Trivially copyable so a copy travels to the device as a kernel argument.
#pragma once

#include <prismspf/config.h>
#include <prismspf/dealii_shim.h>

PRISMS_PF_BEGIN_NAMESPACE

class SimulationTimer {
 public:
  PPF_HD SimulationTimer() {}
  PPF_HD explicit SimulationTimer(double step_size, double start_time = 0.0)
      : current_time(start_time), time_step_size(step_size) {}
  PPF_HD unsigned int get_increment() const { return current_increment; }
  PPF_HD double get_time() const { return current_time; }
  PPF_HD double get_timestep() const { return time_step_size; }
  PPF_HD void increment(double step_size) { current_increment++; current_time += step_size; }
  PPF_HD void increment() { increment(time_step_size); }
  PPF_HD void set_timestep(double s) { time_step_size = s; }
  PPF_HD void set_time(double t) { current_time = t; }
  PPF_HD void set_increment(unsigned int i) { current_increment = i; }
  PPF_HD void reset() { current_increment = 0; current_time = 0.0; }

 private:
  unsigned int current_increment = 0;
  double current_time = 0.0;
  double time_step_size = 0.0;
};

PRISMS_PF_END_NAMESPACE
