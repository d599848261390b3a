/* Stand-in for a Windows CRT header so the reference CPU sources compile with g++. */
#pragma once
