/* Stand-in for a Windows SDK header so the reference CPU sources compile with g++. */
#pragma once
