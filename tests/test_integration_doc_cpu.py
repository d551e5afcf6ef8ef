"""The JNI shim (ressim_gb300/jni/rsg_jni.c) compiles against include/rsg.h,
and the integration guide quotes it verbatim.  There is no JDK here, so a minimal
stand-in declares the few JNI types and JNIEnv functions the shim uses (with
the JNI specification's signatures); the check is that the shim's calls into
the C ABI match the header."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

JNI_STANDIN = r"""
#pragma once
typedef int jint;
typedef long long jlong;
typedef unsigned char jboolean;
typedef double jdouble;
typedef void* jobject;
typedef jobject jclass;
typedef jobject jarray;
typedef jint jsize;
typedef jarray jintArray;
typedef jarray jlongArray;
typedef jarray jdoubleArray;
struct JNINativeInterface_;
typedef const struct JNINativeInterface_* JNIEnv;
struct JNINativeInterface_ {
  void* (*GetPrimitiveArrayCritical)(JNIEnv*, jarray, jboolean*);
  void (*ReleasePrimitiveArrayCritical)(JNIEnv*, jarray, void*, jint);
  void (*SetIntArrayRegion)(JNIEnv*, jintArray, jint, jint, const jint*);
  void (*SetDoubleArrayRegion)(JNIEnv*, jdoubleArray, jint, jint, const jdouble*);
  void (*SetLongArrayRegion)(JNIEnv*, jlongArray, jint, jint, const jlong*);
  jsize (*GetArrayLength)(JNIEnv*, jarray);
};
#define JNIEXPORT
#define JNICALL
#define JNI_ABORT 2
"""


SHIM = os.path.join(ROOT, "ressim_gb300", "jni", "rsg_jni.c")


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_jni_shim_compiles_against_the_header(tmp_path):
    (tmp_path / "jni.h").write_text(JNI_STANDIN)
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-c", "-I", str(tmp_path), "-I",
                        os.path.join(ROOT, "include"), SHIM, "-o", str(tmp_path / "shim.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_doc_quotes_the_shim():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, re.S)
    assert blocks and "rsg_solver_solve" in blocks[0]
    src = open(SHIM).read()
    for b in blocks:
        assert b.strip() in src
