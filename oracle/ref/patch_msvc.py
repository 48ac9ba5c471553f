"""Mechanical MSVC -> GCC rewrite of the reference's Model.cpp into a build directory.

Only constructs GCC rejects are touched; the arithmetic is not. Reads the reference source,
writes the patched copy to the output path (under oracle/_ref, never into the repository):
  x.swap(vector<T>())           -> vector<T>().swap(x)
  v.m128_f32[i]                 -> v[i]                       (GCC vector subscript)
  v.m256_f32[i]                 -> v[i]
  v.m256i_i32[i]                -> ((const int32_t *)&v)[i]   (32-bit lanes, not GCC's 64-bit)
  *(__m256i*)&_mm256_cmp_ps(..) -> _mm256_castps_si256(_mm256_cmp_ps(..))
"""
import re
import sys

src, dst = sys.argv[1], sys.argv[2]
s = open(src, encoding="latin-1").read()
n0 = len(s)
s, a = re.subn(r"(\w+)\.swap\((vector<[^;]*?>)\(\)\);", r"\2().swap(\1);", s)
s, b = re.subn(r"\.m128_f32\[", "[", s)
s, c = re.subn(r"\.m256_f32\[", "[", s)
s, d = re.subn(r"(\w+)\.m256i_i32\[", r"((const int32_t *)&\1)[", s)
s, e = re.subn(r"\*\(__m256i\*\)&(_mm256_cmp_ps\([^;]*?\));", r"_mm256_castps_si256(\1);", s)
open(dst, "w", encoding="latin-1").write(s)
print(f"patched {src}: swap {a}, m128 {b}, m256 {c}, m256i {d}, cmp {e}")
