"""Copies the reference's OpenMP PBF solver and the headers it includes into
oracle/_ref/src/ (git-ignored; it travels to the GPU machine beside the built files) and
patches cpusph.hpp so that it compiles against the current interface (TEST
INFRASTRUCTURE: the benchmark's timed reference arm).

cpu::SphSolver::advance (include/fluid/cpusph.hpp:122-238) declares the return type
std::vector<surface::MeshTriangle<N>> while the base class it overrides requires
fluid::Result<N> (include/fluid/fluid.hpp:228), and its body has no return statement.
The two patches: the declared return type becomes fluid::Result<N>, and the body
ends with `return fluid::Result<N>();` (the solver extracts no surface).  Nothing
else changes.  GLM, which the headers include, is replaced by the project-written
subset in oracle/glm_subset; nanoflann is the reference's vendored copy
(third_party/nanoflann.hpp).

usage: python patch_cpusph.py <reference tree> <output directory>
"""
import os
import sys


def write_if_changed(path, text):
    """Keep the file (and its time stamp) when the content is the same, so that the
    solver is not recompiled on every build."""
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as f:
        f.write(text)


def main(ref, out):
    os.makedirs(out, exist_ok=True)
    inc = os.path.join(ref, "include", "fluid")
    for name in ("fluid.hpp", "geometry.hpp", "curves.h"):
        write_if_changed(os.path.join(out, name), open(os.path.join(inc, name)).read())
    write_if_changed(os.path.join(out, "nanoflann.hpp"), open(os.path.join(ref, "third_party", "nanoflann.hpp")).read())
    src = open(os.path.join(inc, "cpusph.hpp")).read()
    patches = [
        ("std::vector<surface::MeshTriangle<N>> advance(const fluid::Config<N> &config,",
         "fluid::Result<N> advance(const fluid::Config<N> &config,"),
        ("a.particle->velocity = (deltaX * (1.f / config.dt) + a.velocity) * VD;\n\t\t\t}\n",
         "a.particle->velocity = (deltaX * (1.f / config.dt) + a.velocity) * VD;\n\t\t\t}\n"
         "\t\t\treturn fluid::Result<N>();\n"),
    ]
    for old, new in patches:
        if src.count(old) != 1:
            sys.exit(f"patch_cpusph: expected exactly one occurrence of {old!r}")
        src = src.replace(old, new)
    write_if_changed(os.path.join(out, "cpusph.hpp"), src)
    # cpusph.hpp includes the OpenCL solver's header, which the CPU path does not use
    # and which needs OpenCL; an empty stand-in takes its place
    write_if_changed(os.path.join(out, "oclsph.hpp"),
                     "// stand-in: the OpenCL solver is not part of the CPU reference arm\n")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
