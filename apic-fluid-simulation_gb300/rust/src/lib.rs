// The crate root the reference leaves empty (so its benches/fluid_benchmark.rs
// cannot name FLIP::apic); here it exports the simulation module.
#![allow(non_snake_case)]
pub mod apic;
