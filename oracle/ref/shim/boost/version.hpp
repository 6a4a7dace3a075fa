#pragma once
#define BOOST_VERSION 106600
#define BOOST_LIB_VERSION "1_66"
